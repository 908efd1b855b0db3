"""The wave-packet basis with auxiliary decorrelation times and variances
(Basis_bmaux, mapping/src/basis.py:1741-2638) restated in
oracle/basis.py::BMauxOracle against golden vectors produced by the
reference's own numpy class (tests/golden/gen_golden_bmaux.py): lattice,
per-centre decorrelation times, window integrals and time centres, Q, and
the projection and its transpose formed from the reference's own Gx and Gt."""
import os

import numpy as np
import pytest

from oracle.basis import BMauxOracle

GOLD = os.path.join(os.path.dirname(__file__), "golden", "bmaux_golden.npz")
PRM = dict(lmin=60., lmax=300., npsp=3.5, facpsp=1.5, facns=1.2, facnlt=2.0, tdecmin=2., tdecmax=15., factdec=1.3,
           facQ=2.0, norm_time=True, flux=False)


@pytest.fixture(scope="module")
def g():
    return dict(np.load(GOLD))


def aux_sorted(g):
    order = np.argsort(g["aux_lon"], kind="stable")
    return dict(f=g["aux_f"], lat=g["aux_lat"], lon=g["aux_lon"][order], Tdec=g["aux_tdec"][..., order],
                Std=g["aux_std"][..., order])


@pytest.fixture(scope="module")
def o(g):
    lon, lat = np.meshgrid(g["lon"], g["lat"])
    b = BMauxOracle(lon, lat, aux_sorted(g), mask=g["mask"], geo=True, time_ref=float(g["time_ref"]), **PRM)
    b.set_basis(g["time"])
    return b


def test_lattice_times_and_q(g, o):
    assert np.allclose(o.ff, g["ff"], rtol=1e-15, atol=0)
    assert np.array_equal(o.NP, g["NP"])
    assert np.array_equal(np.asarray(o.bounds), g["bounds"])
    for iff in range(o.nf):
        assert np.allclose(o.ENSLAT[iff], g[f"f{iff}_lat"], rtol=1e-14, atol=0)
        assert np.allclose(o.ENSLON[iff], g[f"f{iff}_lon"], rtol=1e-14, atol=0)
        assert np.allclose(o.tdec[iff], g[f"f{iff}_tdec"], rtol=1e-13, atol=0)
        assert np.allclose(o.norm_fact[iff], g[f"f{iff}_norm"], rtol=1e-13, atol=0)
        assert np.array_equal(np.isnan(o.enst[iff]), np.isnan(g[f"f{iff}_enst"]))
        # t0 = -time_ref mod tdec (time_ref ~ 2.3e4 days) turns the last-bit
        # rounding of the interpolated tdec (1e-16, interpolation order) into
        # ~1e-12-day offsets of the time centres
        m = ~np.isnan(g[f"f{iff}_enst"])
        assert np.allclose(o.enst[iff][m], g[f"f{iff}_enst"][m], rtol=0, atol=1e-10)
    assert np.allclose(o.Q, g["q"], rtol=1e-13, atol=0)
    # per-centre times really differ (the aux field varies over the domain)
    assert max(np.ptp(t) for t in o.tdec if t.size) > 0.5


def test_projection_and_transpose(g, o):
    for k in g["times_k"]:
        t = g["time"][k]
        phi = o.operg(t, g["X"])
        adX = o.operg_transpose(t, g[f"t{k}_ad"])
        e1 = np.abs(phi - g[f"t{k}_phi"]).max() / np.abs(g[f"t{k}_phi"]).max()
        e2 = np.abs(adX - g[f"t{k}_adX"]).max() / np.abs(g[f"t{k}_adX"]).max()
        # the time-centre offsets above bound the agreement near 1e-12
        assert e1 < 1e-11 and e2 < 1e-11, (k, e1, e2)


def test_library_host_tables_match_reference(g):
    """The plan's host tables (built by the library in C++, no device)
    against the reference's own class."""
    from vardyn_gb300.basis import BMauxParams, BMauxPlan
    plan = BMauxPlan(g["lon"], g["lat"], g["time"], BMauxParams(aux_sorted(g), time_ref=float(g["time_ref"]), **PRM),
                     land=g["mask"], geographic=True, host_only=True)
    assert plan.nf == g["ff"].size and plan.ntheta == g["theta"].size
    assert np.allclose(plan.theta, g["theta"], rtol=1e-15, atol=0)
    assert plan.nbasis == g["bounds"][-1]
    assert np.allclose(plan.q(), g["q"], rtol=1e-13, atol=0)
    for iff in range(plan.nf):
        ff, _, off, nt, ns = plan.frequency(iff)
        assert abs(ff - g["ff"][iff]) <= 1e-15 * g["ff"][iff]
        assert off == g["bounds"][iff] and ns == g["NP"][iff] and nt == g[f"f{iff}_enst"].shape[1]
        enst, lat, lon = plan.lattice(iff)
        assert np.allclose(lat, g[f"f{iff}_lat"], rtol=1e-14, atol=0)
        assert np.allclose(lon, g[f"f{iff}_lon"], rtol=1e-14, atol=0)
        ref = g[f"f{iff}_enst"]
        assert np.array_equal(np.isnan(enst), np.isnan(ref))
        assert np.allclose(enst[~np.isnan(ref)], ref[~np.isnan(ref)], rtol=0, atol=1e-10)
        td, nrm, n = plan.centres(iff)
        assert np.allclose(td, g[f"f{iff}_tdec"], rtol=1e-13, atol=0)
        assert np.allclose(nrm, g[f"f{iff}_norm"], rtol=1e-13, atol=0)
        assert np.array_equal(n, (~np.isnan(ref)).sum(axis=1))


def test_drop_in_longitude_handling():
    """prepare_aux converts the dataset's longitudes as basis.py:1944-1948
    and sorts them."""
    from vardyn_gb300.basis import Basis_bmaux
    ds = dict(f=[1.0, 2.0], lat=[0.0, 1.0], lon=np.array([350.0, 10.0, 190.0]),
              Tdec=np.arange(12.0).reshape(2, 2, 3), Std=np.ones((2, 2, 3)))
    a = Basis_bmaux.prepare_aux(ds, "-180_180")
    assert np.array_equal(a["lon"], [-170.0, -10.0, 10.0])
    assert np.array_equal(a["Tdec"][0, 0], [2.0, 0.0, 1.0])
    b = Basis_bmaux.prepare_aux(dict(ds, lon=np.array([-20.0, 5.0, 30.0])), "0_360")
    assert np.array_equal(b["lon"], [5.0, 30.0, 340.0])
