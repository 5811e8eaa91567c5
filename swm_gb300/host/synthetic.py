"""Seeded synthetic workloads on the reference's spherical grid.

The workloads are stated in Cartesian terms (cells, dx in metres, beta-plane
f0/beta).  The reference has no Cartesian mode, so they are mapped onto its
lon/lat grid with a radius 1000x Earth's: spans are then a few 1e-3 rad,
cos(lat) = 1 - O(1e-6) and tan(lat)/A ~ 0, i.e. Cartesian to ~1e-6, and the
beta-plane is coriolis_approx = 2 with 2*OMEGA*sin(theta0) = f0 and
2*OMEGA*cos(theta0)/A = beta.  H arrays carry the land of a closed basin
(the reference zeroes the first/last row itself; east/west come from H).

Seeds: numpy PCG64(20260 + workload index) (+ member * 7919 for ensemble
members), drawn in FP64 on the host.
"""
import math
import numpy as np

from .case import MODE_NONE, MODE_NONLINEAR, MODE_LIN_REST

A_BIG = 6.371e9
D2R = float(np.float32(3.14159265358979323846)) / 180.0
DAY = 86400.0


def _base_config(cells_x, cells_y, dx, f0, beta, dt):
    span_x = cells_x * dx / A_BIG / D2R
    span_y = cells_y * dx / A_BIG / D2R
    two_omega = math.hypot(f0, beta * A_BIG)
    theta0 = math.degrees(math.atan2(f0, beta * A_BIG)) if two_omega > 0 else 0.0
    return dict(nx=cells_x + 1, ny=cells_y + 1, mode=MODE_NONLINEAR, lateral_mixing=1, quadratic_friction=0,
                barotropic=0, mixing_kind=0, coriolis_approx=2, tracer_nan_guard=0, damping_additive=0,
                mask_psi_bs=0, dt=dt, G=9.81, Ah=0.0, A=A_BIG, OMEGA=two_omega / 2.0, RHO0=1024.0, lbc=2.0,
                theta0=theta0, lon_s=-span_x / 2, lon_e=span_x / 2, lat_s=-span_y / 2, lat_e=span_y / 2,
                H_overwrite=0.0, ab_chi=0.1, minD=1.0, tau_scale=1.0, bih=0.0, diag_start_ind=0,
                meant_out=2.628e6, tracer=0)


def perturbed_basin(nx, ny, depth, rng, max_inset=3):
    """H (ny, nx): depth inside a closed basin whose boundary cells are moved
    inwards by 0..max_inset cells, independently per boundary cell."""
    H = np.full((ny, nx), float(depth))
    H[:, 0] = 0.0
    H[:, -1] = 0.0
    H[0, :] = 0.0
    H[-1, :] = 0.0
    inset = rng.integers(0, max_inset + 1, size=(4, max(nx, ny)))
    for j in range(ny):
        H[j, :1 + inset[0, j]] = 0.0
        H[j, nx - 1 - inset[1, j]:] = 0.0
    for i in range(nx):
        H[:1 + inset[2, i], i] = 0.0
        H[ny - 1 - inset[3, i]:, i] = 0.0
    return H


def _wind_stream(cfg, amp, ny):
    """tau_x = amp * cos(2*pi*y/L) on the u grid rows, constant in time."""
    lat_u = np.array([j * (cfg['lat_e'] - cfg['lat_s']) / (ny - 1) + cfg['lat_s'] for j in range(ny)]) + \
        (cfg['lat_e'] - cfg['lat_s']) / (2.0 * (ny - 1))
    y = (lat_u - cfg['lat_s']) / (cfg['lat_e'] - cfg['lat_s'])
    prof = amp * np.cos(2.0 * math.pi * y)
    rec = np.repeat(prof[:, None], cfg['nx'], axis=1)[None]
    return dict(type=0, comp=0, omega=0.0, rec1=rec, dt1=0.0, chunksize=100, rec2=None, dt2=0.0)


def empty_case(cfg):
    return {'config': cfg, 'H': None, 'H_missing': None, 'psi_bs': None, 'damping': [], 'streams': [],
            'ic': {}, 'tracers': [], 'diag': []}


def linear_rg(cells_x=256, cells_y=128, seed_index=0, nsteps=10000):
    """Plain linear reduced-gravity SWM: beta-plane (f = beta*y), g' = 0.02,
    H = 200 m, Ah = 1000, Rayleigh 1/(100 d), closed box, Gaussian eta bump
    (0.1 m, 300 km e-folding) at a seed-drawn interior point, AB3 dt = 1800 s."""
    rng = np.random.Generator(np.random.PCG64(20260 + seed_index))
    dx = 25e3
    cfg = _base_config(cells_x, cells_y, dx, 0.0, 2.3e-11, 1800.0)
    cfg.update(mode=MODE_LIN_REST, G=0.02, Ah=1000.0, H_overwrite=200.0, Nt=nsteps)
    case = empty_case(cfg)
    nx, ny = cfg['nx'], cfg['ny']
    H = np.ones((ny, nx))
    H[:, 0] = H[:, -1] = 0.0
    case['H'] = H
    g = 1.0 / (100.0 * DAY)
    case['damping'] = [dict(term=0, type=0, value=g, sl_length=1.0, sl_cutoff=15.0, loc=0, file_data=None),
                       dict(term=1, type=0, value=g, sl_length=1.0, sl_cutoff=15.0, loc=0, file_data=None)]
    cx, cy = rng.uniform(0.25, 0.75) * cells_x * dx, rng.uniform(0.25, 0.75) * cells_y * dx
    x = (np.arange(nx) + 0.5) * dx
    y = (np.arange(ny) + 0.5) * dx
    r2 = (x[None, :] - cx) ** 2 + (y[:, None] - cy) ** 2
    case['ic'] = {'eta': 0.1 * np.exp(-r2 / (300e3) ** 2)}
    return case


def double_gyre(cells=1024, seed_index=1, nsteps=20000, biharmonic=True, dx=5e3, amp=0.1, ah=None,
                rng=None, dt=15.0):
    """Nonlinear single-layer wind-driven double gyre: beta-plane f0 = 1e-4,
    beta = 2e-11, H = 500 m, g = 9.81, tau = amp*cos(2 pi y/L), bottom drag
    1e-7 /s (linear, not divided by H), biharmonic 1e10 m^4/s (extension) or
    Laplacian Ah (reference), perturbed closed coastline, rest, AB3.

    dt defaults to 15 s: at dx = 5 km and H = 500 m the 2-dx gravity wave has
    omega*dt = 2*sqrt(2)*sqrt(gH)*dt/dx = 0.79 for dt = 20 s, outside AB3's
    stability interval on the imaginary axis (|omega*dt| <= 0.72); the run
    blows up after a few hundred steps."""
    if rng is None:
        rng = np.random.Generator(np.random.PCG64(20260 + seed_index))
    cells_x, cells_y = (cells, cells) if np.isscalar(cells) else cells
    cfg = _base_config(cells_x, cells_y, dx, 1e-4, 2e-11, dt)
    cfg.update(mode=MODE_NONLINEAR, G=9.81, Nt=nsteps)
    if biharmonic:
        cfg.update(mixing_kind=1, bih=1e10, Ah=0.0)
    else:
        cfg.update(mixing_kind=0, Ah=500.0 if ah is None else ah)
    case = empty_case(cfg)
    case['H'] = perturbed_basin(cfg['nx'], cfg['ny'], 500.0, rng)
    r = 1e-7
    case['damping'] = [dict(term=0, type=0, value=r, sl_length=1.0, sl_cutoff=15.0, loc=0, file_data=None),
                       dict(term=1, type=0, value=r, sl_length=1.0, sl_cutoff=15.0, loc=0, file_data=None)]
    case['streams'] = [_wind_stream(cfg, amp, cfg['ny'])]
    return case


def ensemble_members(n=256, seed_index=4, nsteps=10000):
    """Ensemble of wind-driven basins of uneven sizes: Nx, Ny log-uniform in
    [64, 512], dx uniform 5-20 km, wind amplitude uniform 0.05-0.2 N/m^2,
    perturbed coastline, Laplacian Ah = 500."""
    out = []
    for m in range(n):
        rng = np.random.Generator(np.random.PCG64(20260 + seed_index + m * 7919))
        cx = int(round(math.exp(rng.uniform(math.log(64), math.log(512)))))
        cy = int(round(math.exp(rng.uniform(math.log(64), math.log(512)))))
        dx = rng.uniform(5e3, 20e3)
        amp = rng.uniform(0.05, 0.2)
        dt = 15.0 * dx / 5e3
        out.append(double_gyre((cx, cy), biharmonic=False, dx=dx, amp=amp, ah=500.0, rng=rng, nsteps=nsteps, dt=dt))
    return out


def _grf(ny, nx, slope, rng):
    """Gaussian random field on (ny, nx) whose Fourier amplitudes fall off as
    |k|^slope (k in cycles per domain, mean removed)."""
    kx = np.fft.fftfreq(nx) * nx
    ky = np.fft.fftfreq(ny) * ny
    k = np.hypot(ky[:, None], kx[None, :])
    amp = np.zeros_like(k)
    amp[k > 0] = k[k > 0] ** slope
    z = rng.standard_normal((ny, nx)) + 1j * rng.standard_normal((ny, nx))
    f = np.fft.ifft2(z * amp).real
    return f - f.mean()


def tracer_flow(cells=2048, dx=2.5e3, seed_index=2, nsteps=5000, depth=100.0, peak_speed=0.5, n_tracers=2,
                kappa=50.0, relax_days=30.0, dt=60.0, flux=1):
    """Two passive tracers in a steady nondivergent flow (prescribed: the SWM
    state is frozen), closed box with a one-cell land rim, uniform depth.

    Streamfunction: Gaussian random field whose kinetic-energy spectrum falls
    off as k^-3 (psi amplitudes ~ k^-3), tapered to zero at the coast and
    scaled to a peak speed of 0.5 m/s; u = -d(psi)/dy, v = d(psi)/dx on the
    C grid, so the discrete divergence vanishes.  Tracers: random fields with
    variance spectrum ~ k^-3 (amplitudes ~ k^-2) mapped to [0, 1]; kappa = 50
    m^2/s; relaxation to the initial field on 30 days; flux 1 = upwind-biased
    (extension), 0 = the reference's centred flux."""
    rng = np.random.Generator(np.random.PCG64(20260 + seed_index))
    cfg = _base_config(cells, cells, dx, 0.0, 0.0, dt)
    cfg.update(mode=MODE_NONE, lateral_mixing=0, Ah=0.0, Nt=nsteps, frozen_flow=1, tracer_flux=flux,
               tracer_nan_guard=1, tracer=1)
    case = empty_case(cfg)
    nx, ny = cfg['nx'], cfg['ny']
    H = np.full((ny, nx), float(depth))
    H[0, :] = H[-1, :] = 0.0
    H[:, 0] = H[:, -1] = 0.0
    case['H'] = H
    psi = _grf(ny, nx, -3.0, rng)
    wy = np.sin(np.pi * np.clip((np.arange(ny) - 1) / (ny - 3), 0, 1)) ** 2
    wx = np.sin(np.pi * np.clip((np.arange(nx) - 1) / (nx - 3), 0, 1)) ** 2
    psi = psi * wy[:, None] * wx[None, :]
    u = np.zeros((ny, nx))
    v = np.zeros((ny, nx))
    u[:-1, :] = -(psi[1:, :] - psi[:-1, :]) / dx
    v[:, :-1] = (psi[:, 1:] - psi[:, :-1]) / dx
    s = peak_speed / max(np.abs(u).max(), np.abs(v).max())
    case['ic'] = {'u': u * s, 'v': v * s}
    for t in range(n_tracers):
        c = _grf(ny, nx, -2.0, rng)
        c = (c - c.min()) / (c.max() - c.min())
        case['tracers'].append(dict(varid='C%d' % t, kappa_h=kappa, cons=0.0, gamma_c=1.0 / (relax_days * DAY),
                                    field_C=c, field_C0=c.copy(), field_gamma_C=None, field_cons=None))
    return case


def _smooth_field(ny, nx, corr_cells, rng):
    """Unit-variance Gaussian random field with a Gaussian correlation of
    corr_cells grid cells (white noise filtered in Fourier space)."""
    fy = np.fft.fftfreq(ny)[:, None]
    fx = np.fft.fftfreq(nx)[None, :]
    filt = np.exp(-2.0 * (np.pi * corr_cells) ** 2 * (fx ** 2 + fy ** 2))
    f = np.fft.ifft2(np.fft.fft2(rng.standard_normal((ny, nx))) * filt).real
    return (f - f.mean()) / f.std()


HELMHOLTZ_LAMBDA = 1.6e-12


def helmholtz_case(cells=4096, dx=5e3, seed_index=3, lam=HELMHOLTZ_LAMBDA):
    """Barotropic streamfunction problem div(H^-1 grad psi) - lam psi = rhs.

    Depth: exp(log(1000 m) + g) with g a unit Gaussian random field of 200 km
    correlation, clipped to 50-5000 m.  Coast: land where a second random
    field (400 km correlation) exceeds its 85th percentile, plus the outer
    frame (psi = 0 on land).  rhs: wind-curl-like random field of 500 km
    correlation with standard deviation 1e-10, 0 on land.  lam = 1.6e-12 (per
    m^3) keeps the Jacobi spectral radius near 0.9995 where H is shallowest,
    so the best relaxation factor lies inside 1.8-1.99.
    Returns dict(H, ocean (int8), rhs, dx, dy, lam)."""
    rng = np.random.Generator(np.random.PCG64(20260 + seed_index))
    n = cells
    g = _smooth_field(n, n, 200e3 / dx, rng)
    H = np.clip(np.exp(np.log(1000.0) + g), 50.0, 5000.0)
    land = _smooth_field(n, n, 400e3 / dx, rng)
    ocean = (land <= np.quantile(land, 0.85)).astype(np.int8)
    ocean[0, :] = ocean[-1, :] = 0
    ocean[:, 0] = ocean[:, -1] = 0
    rhs = 1e-10 * _smooth_field(n, n, 500e3 / dx, rng) * ocean
    return dict(H=H, ocean=ocean, rhs=rhs, dx=dx, dy=dx, lam=lam)
