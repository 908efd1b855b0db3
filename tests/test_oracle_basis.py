"""Gaussian space-time basis: the oracle against the reference's analytic
definitions, and the library's host-side lattice / time-weight builder
against the oracle (no GPU: the plan is built with host_only)."""
import numpy as np
import pytest

from oracle.basis import Gauss3dOracle, MultiOracle, mywindow


def _planar(ny=60, nx=70, dx=5.0):
    x = np.arange(nx) * dx
    y = 2.0 + np.arange(ny) * dx
    return np.meshgrid(x, y)


def test_single_centre_footprint_is_cos2_product():
    X2, Y2 = _planar()
    o = Gauss3dOracle(X2, Y2, sigma_D=60, sigma_T=5, facns=2, facnlt=2)
    o.set_basis(np.arange(0, 10.01, 0.5))
    t = 2.5
    act = o.time_weights(t)
    assert act, "no active time centre"
    it, g = act[0]
    c = o.Nx // 2 + 3
    X = np.zeros(o.nbasis)
    X[it * o.Nx + c] = 1.0
    phi = o.operg(t, X)
    dx = X2 - o.ENSLON[c]
    dy = Y2 - o.ENSLAT[c]
    inside = (np.abs(dx) <= 60) & (np.abs(dy) <= 60)
    expect = np.where(inside, mywindow(dx / 60) * mywindow(dy / 60), 0.0) * g
    assert np.abs(phi - expect).max() < 1e-15


def test_time_weights_normalised_window():
    X2, Y2 = _planar(10, 10)
    o = Gauss3dOracle(X2, Y2, sigma_D=60, sigma_T=4, facns=2, facnlt=2, normalize_fact=True)
    o.set_basis(np.arange(0, 12.01, 1.0))
    # the trapezoid integral of cos^2 over [-sigma_T, sigma_T] is close to sigma_T
    assert abs(o.norm_fact - 4.0) < 1e-2
    for t in (0.0, 3.0, 7.0):
        for it, f in o.time_weights(t):
            dt = t - o.ENST[it]
            assert abs(dt) < 4
            assert abs(f - mywindow(dt / 4) / o.norm_fact) < 1e-15


@pytest.mark.parametrize("geo", [False, True])
def test_oracle_transpose_identity_with_land(geo):
    if geo:
        lon, lat = np.meshgrid(-40 + np.arange(50) * 0.06, 20 + np.arange(40) * 0.06)
    else:
        lon, lat = _planar(40, 50)
    land = np.zeros(lon.shape, bool)
    land[10:15, 20:30] = True
    comps = [Gauss3dOracle(lon, lat, 90, 6, 2, 2, mask=land, geo=geo),
             Gauss3dOracle(lon, lat, 50, 3, 1.5, 1, mask=land, geo=geo, time_spinup=2.0)]
    m = MultiOracle(comps)
    time = np.arange(0, 8.01, 0.25)
    m.set_basis(time)
    rng = np.random.default_rng(0)
    X = rng.standard_normal(m.nbasis)
    a = rng.standard_normal(lon.shape)
    for t in (0.0, 1.25, 5.5):
        phi = m.operg(t, X)
        assert np.all(phi[land] == 0)
        lhs = np.sum(phi * a)
        rhs = np.dot(X, m.operg_transpose(t, a))
        assert abs(lhs - rhs) <= 1e-12 * max(abs(lhs), 1.0)


def test_multi_is_sum_of_components():
    X2, Y2 = _planar(30, 30)
    comps = [Gauss3dOracle(X2, Y2, 40, 5, 2, 2), Gauss3dOracle(X2, Y2, 70, 8, 1, 2)]
    m = MultiOracle(comps)
    time = np.arange(0, 6.01, 1.0)
    m.set_basis(time)
    X = np.random.default_rng(1).standard_normal(m.nbasis)
    phi = m.operg(3.0, X)
    ref = comps[0].operg(3.0, X[m.slices[0]]) + comps[1].operg(3.0, X[m.slices[1]])
    assert np.array_equal(phi, ref)


@pytest.mark.parametrize("geo", [False, True])
def test_library_lattice_matches_oracle(geo):
    """The C++ table builder reproduces the reference lattice (NumPy arange
    sequences), the prior std and the active time weights exactly."""
    from vardyn_gb300 import build
    from vardyn_gb300.basis import BasisPlan, Gauss3dParams
    build.build()
    if geo:
        xc, yc = -70 + np.arange(120) * 0.05, 30 + np.arange(90) * 0.05
    else:
        xc, yc = np.arange(100) * 5.0, 3.0 + np.arange(80) * 5.0
    time = np.arange(0, 20.01, 0.25)
    comps = [Gauss3dParams(100, 5, facns=2, facnlt=2, sigma_Q=0.1),
             Gauss3dParams(60, 10, facns=1.5, facnlt=3, sigma_Q=0.2, time_spinup=3.0),
             Gauss3dParams(80, 4, facns=1, facnlt=1, sigma_Q=0.3, flux=True, normalize_fact=False)]
    plan = BasisPlan(xc, yc, time, comps, geographic=geo, host_only=True)
    lon, lat = np.meshgrid(xc, yc)
    orc = MultiOracle([Gauss3dOracle(lon, lat, c.sigma_D, c.sigma_T, c.facns, c.facnlt, c.sigma_Q,
                                     normalize_fact=c.normalize_fact, time_spinup=c.time_spinup,
                                     flux=c.flux, geo=geo) for c in comps])
    _, Q = orc.set_basis(time)
    assert plan.nbasis == orc.nbasis
    assert np.array_equal(plan.q(), Q)
    for c, o in enumerate(orc.comps):
        off, nt, ns = plan.component(c)
        assert off == orc.slices[c].start and nt == o.ENST.size and ns == o.Nx
        enst, la, lo = plan.lattice(c)
        assert np.array_equal(enst, o.ENST)
        assert np.array_equal(la, o.ENSLAT)
        assert np.array_equal(lo, o.ENSLON)
        for k, t in enumerate(time):
            got = plan.time_weights(k, c)
            want = o.time_weights(t)
            assert [i for i, _ in got] == [i for i, _ in want]
            assert np.allclose([w for _, w in got], [w for _, w in want], rtol=0, atol=1e-15)


def test_oracle_basis_4dvar_gradient_central_differences():
    """The oracle's reduced-basis 4D-Var gradient (forcing added at every
    model call end, adjoint accumulated per basis interval) against central
    differences of its own cost."""
    from oracle.fourdvar import ObsSet, cost_and_grad_basis
    from oracle.qg1l import QgmOracle
    from vardyn_gb300.synthetic import kminus3_ssh, satellite_tracks
    ny, nx, dx, dt, nstep, nck = 24, 28, 5e3, 900.0, 10, 4
    rng = np.random.default_rng(2)
    xk, yk = np.arange(nx) * 5.0, np.arange(ny) * 5.0
    lon, lat = np.meshgrid(xk, yk)
    basis = MultiOracle([Gauss3dOracle(lon, lat, 40, 0.1, 1.0, 2.0, 0.05)])
    tb = np.arange(0, nstep * dt + nck * dt, nck * dt) / 86400
    Xb, Q = basis.set_basis(tb)
    x, y, st = satellite_tracks(ny, nx, dx, dx, nstep, 120, rng, spacing_km=6.0)
    st[:5] = 0
    obs = ObsSet(x, y, st, 0.1 * rng.standard_normal(x.size), np.full(x.size, 0.03), ny, nx, dx, dx)
    ref = QgmOracle(dx=np.full((ny, nx), dx), dy=np.full((ny, nx), dx), dt=dt, c=2.7, f=1e-4,
                    time_scheme="rk2")
    h0 = kminus3_ssh(ny, nx, dx, dx, rng, rms=0.1, cutoff_km=20.0)
    hb = np.zeros((ny, nx))
    X0 = rng.standard_normal(basis.nbasis)
    J, G = cost_and_grad_basis(ref, basis, tb, X0, Xb, Q, h0, hb, nstep, nck, obs)
    d = rng.standard_normal(X0.size)
    gd = G.dot(d)
    errs = []
    for eps in (1e-3, 1e-4, 1e-5):
        Jp = cost_and_grad_basis(ref, basis, tb, X0 + eps * d, Xb, Q, h0, hb, nstep, nck, obs)[0]
        Jm = cost_and_grad_basis(ref, basis, tb, X0 - eps * d, Xb, Q, h0, hb, nstep, nck, obs)[0]
        errs.append(abs((Jp - Jm) / (2 * eps) - gd) / abs(gd))
    assert min(errs) < 1e-7, errs


@pytest.mark.parametrize("geo,land", [(False, False), (True, False), (False, True), (True, True)])
def test_library_bm_tables_match_oracle(geo, land):
    """Wave-packet basis: frequencies, directions, lattices (with masked
    centres dropped), time centres, Q and time weights of the C++ builder
    equal the oracle's restatement of Basis_bm exactly."""
    from vardyn_gb300 import build
    from vardyn_gb300.basis import BMParams, BMPlan
    from oracle.basis import BMOracle
    build.build()
    if geo:
        xc, yc = -60 + np.arange(110) * 0.05, 25 + np.arange(95) * 0.05
    else:
        xc, yc = np.arange(100) * 5.0, 2.0 + np.arange(90) * 5.0
    mask = None
    if land:
        mask = np.zeros((yc.size, xc.size), bool)
        mask[:30, :40] = True
    time = np.arange(0, 10.01, 0.25)
    kw = dict(lmin=60, lmax=300, npsp=3.5, facpsp=1.5, lmeso=150, tmeso=10, time_ref=3.3, facns=1.2, facnlt=2.0)
    plan = BMPlan(xc, yc, time, BMParams(**kw), land=mask, geographic=geo, host_only=True)
    lon, lat = np.meshgrid(xc, yc)
    o = BMOracle(lon, lat, mask=mask, geo=geo, **kw)
    _, Q = o.set_basis(time)
    assert plan.nbasis == o.nbasis and plan.nf == o.nf and plan.ntheta == o.ntheta
    assert np.array_equal(plan.theta, o.theta)
    assert np.array_equal(plan.q(), Q)
    for iff in range(o.nf):
        ff, td, off, nt, ns = plan.frequency(iff)
        assert ff == o.ff[iff] and td == o.tdec[iff] and off == o.bounds[iff]
        enst, la, lo = plan.lattice(iff)
        assert np.array_equal(enst, o.enst[iff])
        assert np.array_equal(la, o.ENSLAT[iff]) and np.array_equal(lo, o.ENSLON[iff])
        for k in range(0, time.size, 5):
            got, want = plan.time_weights(k, iff), o.time_weights(iff, time[k])
            assert [i for i, _ in got] == [i for i, _ in want]
            assert np.allclose([w for _, w in got], [w for _, w in want], rtol=0, atol=1e-15)


def test_bm_oracle_transpose_identity():
    from oracle.basis import BMOracle
    lon, lat = np.meshgrid(np.arange(70) * 5.0, np.arange(60) * 5.0)
    mask = np.zeros(lon.shape, bool)
    mask[10:20, 30:45] = True
    o = BMOracle(lon, lat, lmin=60, lmax=250, lmeso=150, tmeso=10, mask=mask)
    o.set_basis(np.arange(0, 6.01, 0.5))
    rng = np.random.default_rng(2)
    X = rng.standard_normal(o.nbasis)
    a = rng.standard_normal(lon.shape)
    for t in (0.0, 2.5, 6.0):
        phi = o.operg(t, X)
        assert np.all(phi[mask] == 0)
        lhs, rhs = np.sum(phi * a), np.dot(X, o.operg_transpose(t, a))
        assert abs(lhs - rhs) <= 1e-12 * max(abs(lhs), 1.0)


@pytest.mark.parametrize("geo", [False, True])
def test_wavelet_host_tables_match_oracle(geo):
    """Wavelet basis (Basis_wavelet3d): lattice and time centres equal the
    oracle's exactly, time weights and Q to rounding."""
    from oracle.basis import WaveletOracle
    from vardyn_gb300.basis import WaveletParams, WaveletPlan
    if geo:
        x = 5.0 + np.arange(40) * 0.08
        y = 35.0 + np.arange(36) * 0.07
        prm = dict(npsp=3.5, facpsp=1.5, facnst=1., lmin=60., lmax=250., tmin=3., tmax=15., sigma_Q=0.02)
    else:
        x = np.arange(60) * 8.0
        y = np.arange(50) * 8.0
        prm = dict(npsp=3.5, facpsp=1.5, facnst=1.2, lmin=60., lmax=250., tmin=3., tmax=15., sigma_Q=0.02)
    land = np.zeros((y.size, x.size), bool)
    land[10:20, 12:25] = True
    time = np.arange(0, 30, 0.25)
    pl = WaveletPlan(x, y, time, WaveletParams(**prm), land=land, geographic=geo, host_only=True)
    X2, Y2 = np.meshgrid(x, y)
    o = WaveletOracle(X2, Y2, mask=land, geo=geo, **prm)
    _, Q = o.set_basis(time)
    assert (pl.nbasis, pl.nf, pl.ntheta) == (o.nbasis, o.nf, o.ntheta)
    for iff in range(o.nf):
        enst, lat, lon = pl.lattice(iff)
        assert np.array_equal(enst, o.enst[iff])
        assert np.array_equal(lat, o.ENSLAT[iff]) and np.array_equal(lon, o.ENSLON[iff])
    for k in range(0, time.size, 7):
        for iff in range(o.nf):
            a, b = pl.time_weights(k, iff), o.time_weights(iff, time[k])
            assert [i for i, _ in a] == [i for i, _ in b]
            assert all(abs(u[1] - v[1]) <= 1e-14 for u, v in zip(a, b))
    assert np.array_equal(pl.q(), Q)
