"""QG 1.5-layer model with passive tracers on the GPU (vd_qgtrac_step,
drop-in Qgm_trac.step) against the reference's own Qgm_trac outputs
(tests/golden/gen_golden_trac.py) and the float64 oracle."""
import os

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(__file__), "golden", "qgtrac_golden.npz")


@pytest.fixture(scope="module", autouse=True)
def built():
    from vardyn_gb300 import build
    build.build()


@pytest.fixture(scope="module")
def g():
    return dict(np.load(GOLD))


def _rel(a, b):
    m = ~np.isnan(b)
    assert np.array_equal(np.isnan(a), np.isnan(b))
    return float(np.abs(a[m] - b[m]).max() / np.abs(b[m]).max())


def _case_a(g, cls, **kw):
    return cls(dx=g["a_dx"], dy=g["a_dy"], dt=900.0, SSH=g["a_ssh"], c=2.7, g=9.81, f=g["a_f"],
               time_scheme=kw.pop("time_scheme", "Euler"), Kdiffus=30.0, Kdiffus_trac=10.0, bc_trac="OBC",
               mdt=g["a_mdt"], **kw)


def test_euler_two_tracers_open_boundaries_matches_reference(g):
    from vardyn_gb300.model_qg1l.jqgm import Qgm_trac
    m = _case_a(g, Qgm_trac, dtype="float64")
    assert _rel(m.step(g["a_X0"], g["a_Xb"], nstep=4), g["a_X1"]) < 1e-11


def test_rk2_dirichlet_relaxation_no_pv_advection_matches_reference(g):
    from vardyn_gb300.model_qg1l.jqgm import Qgm_trac
    m = Qgm_trac(dx=g["b_dx"], dy=g["b_dx"], dt=600.0, SSH=g["b_ssh"], c=2.5, g=9.81, f=1.0e-4,
                 time_scheme="rk2", Wbc=g["b_wbc"], Kdiffus=None, Kdiffus_trac=5.0, bc_trac="dirichlet",
                 advect_pv=False, dtype="float64")
    assert _rel(m.step(g["b_X0"], g["b_Xb"], nstep=3), g["b_X1"]) < 1e-11


def test_rk2_ssh_alone_matches_reference(g):
    from vardyn_gb300.model_qg1l.jqgm import Qgm_trac
    m = Qgm_trac(dx=g["c_dx"], dy=g["c_dx"], dt=900.0, SSH=g["c_ssh"], c=2.7, g=9.81, f=1.0e-4,
                 time_scheme="rk2", Kdiffus=15.0, dtype="float64")
    assert _rel(m.step(g["c_ssh"], g["c_hb"], nstep=3), g["c_h1"]) < 1e-11


def test_rk4_extension_matches_oracle(g):
    from oracle.qg1l_trac import QgmTracOracle
    from vardyn_gb300.model_qg1l.jqgm import Qgm_trac
    m = _case_a(g, Qgm_trac, time_scheme="rk4", dtype="float64")
    o = _case_a(g, QgmTracOracle, time_scheme="rk4")
    assert _rel(m.step(g["a_X0"], g["a_Xb"], nstep=5), o.step(g["a_X0"], g["a_Xb"], nstep=5)) < 1e-11


def test_float32_matches_reference(g):
    from vardyn_gb300.model_qg1l.jqgm import Qgm_trac
    m = _case_a(g, Qgm_trac, dtype="float32")
    assert _rel(m.step(g["a_X0"], g["a_Xb"], nstep=4), g["a_X1"]) < 1e-4


def test_batched_windows_equal_single_windows(g):
    """Three windows in one call equal three calls (the windows are
    independent); zero steps give the input with NaN on land."""
    from vardyn_gb300.model_qg1l.jqgm import Qgm_trac
    m = _case_a(g, Qgm_trac, time_scheme="rk2", dtype="float64")
    rng = np.random.default_rng(4)
    X0 = np.stack([g["a_X0"] + 0.02 * b * rng.standard_normal(g["a_X0"].shape) for b in range(3)])
    Xb = np.stack([g["a_Xb"]] * 3)
    dev = lambda a: torch.as_tensor(a, device="cuda")
    h1, c1 = m.step_windows(dev(X0[:, 0]), dev(X0[:, 1:]), dev(Xb[:, 0]), dev(Xb[:, 1:]), nstep=3)
    for b in range(3):
        one = m.step(X0[b], Xb[b], nstep=3)
        assert _rel(h1[b].cpu().numpy(), one[0]) < 1e-13
        assert _rel(c1[b].cpu().numpy(), one[1:]) < 1e-13
    z = m.step(g["a_X0"], g["a_Xb"], nstep=0)
    land = np.isnan(g["a_X1"][0])
    assert np.all(np.isnan(z[:, land]))
    assert np.allclose(z[:, ~land], g["a_X0"][:, ~land], rtol=0, atol=1e-15)


# ---- tangent linear and adjoint (jqgm.py:2141-2151) against the oracle's,
# which central differences of the reference-pinned step and a dot-product
# test check (tests/test_oracle_qg1l_trac.py)

def _ad_kw(g, key):
    if key == "a":
        kw = dict(dx=g["a_dx"], dy=g["a_dy"], dt=900.0, SSH=g["a_ssh"], c=2.7, g=9.81, f=g["a_f"],
                  time_scheme="Euler", Kdiffus=30.0, Kdiffus_trac=10.0, bc_trac="OBC", mdt=g["a_mdt"])
        X0, Xb = g["a_X0"], g["a_Xb"]
    elif key == "b":
        kw = dict(dx=g["b_dx"], dy=g["b_dx"], dt=600.0, SSH=g["b_ssh"], c=2.5, g=9.81, f=1.0e-4, time_scheme="rk2",
                  Wbc=g["b_wbc"], Kdiffus_trac=5.0, bc_trac="dirichlet", advect_pv=False)
        X0, Xb = g["b_X0"], g["b_Xb"]
    elif key == "rk2obc":
        kw = dict(dx=g["a_dx"], dy=g["a_dy"], dt=900.0, SSH=g["a_ssh"], c=2.7, g=9.81, f=g["a_f"],
                  time_scheme="rk2", Kdiffus=30.0, Kdiffus_trac=10.0, bc_trac="OBC")
        X0, Xb = g["a_X0"], g["a_Xb"]
    elif key == "rk4":
        kw = dict(dx=g["a_dx"], dy=g["a_dy"], dt=900.0, SSH=g["a_ssh"], c=2.7, g=9.81, f=g["a_f"],
                  time_scheme="rk4", Kdiffus_trac=10.0, bc_trac="OBC", mdt=g["a_mdt"])
        X0, Xb = g["a_X0"], g["a_Xb"]
    else:
        kw = dict(dx=g["c_dx"], dy=g["c_dx"], dt=900.0, SSH=g["c_ssh"], c=2.7, g=9.81, f=1.0e-4, time_scheme="rk2",
                  Kdiffus=15.0)
        X0, Xb = g["c_ssh"], g["c_hb"]
    return kw, np.nan_to_num(np.asarray(X0, dtype=np.float64)), np.asarray(Xb, dtype=np.float64)


def _relmax(a, b):
    return float(np.abs(a - b).max() / np.abs(b).max())


@pytest.mark.parametrize("key", ["a", "b", "rk2obc", "rk4", "c"])
def test_tangent_and_adjoint_match_oracle(g, key):
    from oracle.qg1l_trac import QgmTracTLAD
    from vardyn_gb300.model_qg1l.jqgm import Qgm_trac
    kw, X0, Xb = _ad_kw(g, key)
    o = QgmTracTLAD(**kw)
    m = Qgm_trac(dtype="float64", **kw)
    rng = np.random.default_rng(41)
    d = rng.standard_normal(X0.shape) * 1e-2
    y = rng.standard_normal(X0.shape)
    y[..., o.ind0] = np.nan                    # NaN on land, as a step leaves it
    tl_ref, tl = o.step_tgl(d, X0, Xb, 3), m.step_tgl(d, X0, Xb, nstep=3)
    ad_ref, ad = o.step_adj(y, X0, Xb, 3), m.step_adj(y, X0, Xb, nstep=3)
    et, ea = _relmax(tl, tl_ref), _relmax(ad, ad_ref)
    print(f"\nQgm_trac {key}: tangent vs oracle {et:.1e}, adjoint vs oracle {ea:.1e}")
    assert et < 1e-10 and ea < 1e-10


def test_dot_product_and_batched_windows(g):
    """<J d, y> = <d, J^T y> to 1e-12 on the GPU, and three windows in one
    call equal three single calls for both the tangent and the adjoint."""
    from vardyn_gb300.model_qg1l.jqgm import Qgm_trac
    kw, X0, Xb = _ad_kw(g, "rk2obc")
    m = Qgm_trac(dtype="float64", **kw)
    rng = np.random.default_rng(42)
    d = rng.standard_normal(X0.shape)
    y = rng.standard_normal(X0.shape)
    tl, ad = m.step_tgl(d, X0, Xb, nstep=4), m.step_adj(y, X0, Xb, nstep=4)
    lhs, rhs = float(np.sum(tl * y)), float(np.sum(d * ad))
    assert abs(lhs - rhs) <= 1e-12 * abs(lhs)
    dev = lambda a: torch.as_tensor(np.ascontiguousarray(a), device="cuda")
    Xs = np.stack([X0 + 0.01 * b * rng.standard_normal(X0.shape) for b in range(3)])
    Ds = rng.standard_normal(Xs.shape)
    XB = np.stack([Xb] * 3)
    th, tc = m.step_tgl_windows(dev(Ds[:, 0]), dev(Ds[:, 1:]), dev(Xs[:, 0]), dev(Xs[:, 1:]), dev(XB[:, 0]),
                                dev(XB[:, 1:]), nstep=2)
    ah, ac = m.step_adj_windows(dev(Ds[:, 0]), dev(Ds[:, 1:]), dev(Xs[:, 0]), dev(Xs[:, 1:]), dev(XB[:, 0]),
                                dev(XB[:, 1:]), nstep=2)
    for b in range(3):
        t1 = m.step_tgl(Ds[b], Xs[b], Xb, nstep=2)
        a1 = m.step_adj(Ds[b], Xs[b], Xb, nstep=2)
        assert _relmax(th[b].cpu().numpy(), t1[0]) < 1e-13 and _relmax(tc[b].cpu().numpy(), t1[1:]) < 1e-13
        assert _relmax(ah[b].cpu().numpy(), a1[0]) < 1e-13 and _relmax(ac[b].cpu().numpy(), a1[1:]) < 1e-13


def test_float32_tangent_and_adjoint(g):
    from oracle.qg1l_trac import QgmTracTLAD
    from vardyn_gb300.model_qg1l.jqgm import Qgm_trac
    kw, X0, Xb = _ad_kw(g, "rk2obc")
    o, m = QgmTracTLAD(**kw), Qgm_trac(dtype="float32", **kw)
    rng = np.random.default_rng(43)
    d = rng.standard_normal(X0.shape) * 1e-2
    for got, ref in ((m.step_tgl(d, X0, Xb, nstep=3), o.step_tgl(d, X0, Xb, 3)),
                     (m.step_adj(d, X0, Xb, nstep=3), o.step_adj(d, X0, Xb, 3))):
        err = np.linalg.norm(got - ref) / np.linalg.norm(ref)
        print(f"\nQgm_trac float32 rel-L2 vs float64 oracle: {err:.2e}")
        assert err < 1e-4
