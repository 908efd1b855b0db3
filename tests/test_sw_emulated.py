"""The shallow-water library (vardyn_gb300/csrc/vd_sw.cu with the Neumann
solve of vd_neumann.cu) run on the CPU: the two source files are compiled by
g++ under the host emulation of tests/host_emulation (every kernel body runs
once per thread of its grid, or once per block for the solve's
barrier-separated block loops), and the library's C ABI is called on host
buffers.

The spectral barotropic filter is checked against the reference's own outputs
(tests/golden/swfilter_golden.npz: the solve, the right-hand side with the
filter, a 3-step run), against the oracle (oracle/sw.py) on a non-uniform
grid with 3 layers and 2 batch members, and for the tangent-linear (central
differences) and the adjoint (dot products, including the cotangent of H).
Open boundaries are checked against the reference's own outputs
(tests/golden/swobc_golden.npz), the model without either against
tests/golden/sw_golden.npz. The same sources run on the GPU in
tests/test_gpu_sw_filter.py and tests/test_gpu_sw.py."""
import ctypes
import os
import shutil
import sys
import types

import numpy as np
import pytest

from oracle.sw import SWOracle
from vardyn_gb300 import _lib

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = os.path.join(HERE, "golden", "swfilter_golden.npz")
DP = ctypes.POINTER(ctypes.c_double)


@pytest.fixture(scope="module")
def emu(tmp_path_factory):
    if shutil.which("g++") is None:
        pytest.skip("g++ is not installed")
    sys.path.insert(0, os.path.join(HERE, "host_emulation"))
    import build_emu
    lib = ctypes.CDLL(build_emu.build(str(tmp_path_factory.mktemp("sw_filter_emu"))))
    for name, (res, args) in _lib.SIGNATURES.items():
        if hasattr(lib, name):
            fn = getattr(lib, name)
            fn.restype, fn.argtypes = res, args
    return lib


@pytest.fixture(scope="module")
def g():
    return dict(np.load(GOLD))


def rel(a, b):
    return np.abs(np.asarray(a) - b).max() / np.abs(b).max()


def ok(status, what):
    assert status == 0, f"{what}: {_lib._STATUS.get(status, status)}"


def ptr(a):
    return None if a is None else ctypes.c_void_p(a.ctypes.data)


class Plan:
    """A vd_sw_plan of the emulated library from the reference's param keys."""

    def __init__(self, lib, prm, dtype=np.float64, bf_lambd=None, H_wind=None):
        self.lib, self.dtype = lib, dtype
        nx, ny, nl = prm["nx"], prm["ny"], prm["nl"]
        self.nx, self.ny, self.nl = nx, ny, nl
        keep = self._keep = []

        def arr(a, shape=None):
            a = np.asarray(a, dtype=np.float64)
            if shape is not None:
                a = np.broadcast_to(a, shape)
            a = np.ascontiguousarray(a)
            keep.append(a)
            return a.ctypes.data_as(DP)

        d = _lib.VdSwDesc()
        d.nx, d.ny, d.nl = nx, ny, nl
        d.dtype = _lib.VD_F64 if dtype == np.float64 else _lib.VD_F32
        d.dx_host, d.dy_host = arr(prm["dx"], (nx, ny)), arr(prm["dy"], (nx, ny))
        d.f_host = arr(prm["f"])
        H = np.asarray(prm["H"], dtype=np.float64)
        if H.size == nl:
            d.H_spatial, d.H_host = 0, arr(H.reshape(nl))
        else:
            d.H_spatial, d.H_host = 1, arr(H.reshape(nl, nx, ny))
        d.g_prime_host = arr(np.asarray(prm["g_prime"]).reshape(nl))
        d.slip_coef = prm.get("slip_coef", 1.0)
        d.bottom_drag_coef = prm.get("bottom_drag_coef", 0.0)
        d.rho_water, d.h_min, d.h_min_sharpness = 1025.0, prm.get("h_min", 0.1), 10.0
        d.visc_coef, d.diff_coef = prm.get("visc_coef", 0.0), prm.get("diff_coef", 0.0)
        d.dt, d.sponge_coef = prm["dt"], prm.get("sponge_coef", 0.0)
        d.forcing_momentum = 1 if prm.get("forcing_momentum") == "mass_consistent" else 0
        if prm.get("mask") is not None:
            d.mask_host = arr(prm["mask"], (nx, ny))
        if prm.get("h_wind") is not None:
            d.h_wind_mode, d.h_wind_scalar = 1, float(prm["h_wind"])
        for name, shape in (("taux", (nx - 1, ny)), ("tauy", (nx, ny - 1))):
            if np.ndim(prm[name]) == 0:
                setattr(d, name + "_scalar", float(prm[name]))
            else:
                setattr(d, name + "_host", arr(prm[name], shape))
        for name, shape in (("sponge_u", (nx + 1, ny)), ("sponge_v", (nx, ny + 1)), ("sponge_h", (nx, ny))):
            if prm.get(name) is not None:
                setattr(d, name + "_host", arr(np.asarray(prm[name]).reshape(shape)))
        if H_wind is not None:
            # the wind depth of a model stepped with a perturbed H stays its own (sw.py:622-630)
            d.Hwind_host = arr(np.asarray(H_wind, dtype=np.float64).reshape(nl, -1)[0], (nx, ny))
        d.barotropic_filter = 1 if prm.get("barotropic_filter") else 0
        d.flag_obc = 1 if prm.get("flag_obc") else 0
        if bf_lambd is not None:
            lam = np.asarray(bf_lambd, dtype=np.float64)
            if lam.size == 1:
                d.bf_lambd_host, d.bf_lambd_spatial = arr(lam.reshape(1)), 0
            else:
                d.bf_lambd_host, d.bf_lambd_spatial = arr(lam.reshape(nx, ny)), 1
        h = ctypes.c_void_p()
        ok(lib.vd_sw_plan_create(ctypes.byref(h), ctypes.byref(d)), "vd_sw_plan_create")
        self.h = h

    def __del__(self):
        if getattr(self, "h", None) is not None:
            self.lib.vd_sw_plan_destroy(self.h)

    def ws(self, B, nstep):
        return np.zeros(self.lib.vd_sw_workspace_bytes(self.h, B, nstep) + 256, dtype=np.uint8)

    def c(self, a):
        return np.ascontiguousarray(a, dtype=self.dtype)

    def shapes(self, B):
        nx, ny, nl = self.nx, self.ny, self.nl
        return (B, nl, nx + 1, ny), (B, nl, nx, ny + 1), (B, nl, nx, ny)

    def step(self, u0, v0, h0, nstep, ub=None, vb=None, hb=None, Fu=None, Fv=None, Fh=None, taux=None, tauy=None):
        B = u0.shape[0]
        ins = [None if a is None else self.c(a) for a in (u0, v0, h0, ub, vb, hb, Fu, Fv, Fh, taux, tauy)]
        out = [np.empty(s, self.dtype) for s in self.shapes(B)]
        w = self.ws(B, nstep)
        a = list(map(ptr, ins))
        ok(self.lib.vd_sw_step(self.h, B, *a[:3], nstep, *a[3:], *map(ptr, out), ptr(w), w.nbytes, None),
           "vd_sw_step")
        return out

    def rhs(self, u, v, h, taux=None, tauy=None):
        B = u.shape[0]
        ins = [None if a is None else self.c(a) for a in (u, v, h, taux, tauy)]
        out = [np.empty(s, self.dtype) for s in self.shapes(B)]
        w = self.ws(B, 0)
        ok(self.lib.vd_sw_rhs(self.h, B, *map(ptr, ins), *map(ptr, out), ptr(w), w.nbytes, None), "vd_sw_rhs")
        return out

    def tgl(self, x, dx, nstep):
        B = x[0].shape[0]
        x, dx = [self.c(a) for a in x], [self.c(a) for a in dx]
        out = [np.empty(s, self.dtype) for s in self.shapes(B)]
        w = self.ws(B, nstep)
        ok(self.lib.vd_sw_step_tgl(self.h, B, *map(ptr, x), *map(ptr, dx), nstep, None, None, None, None, None, None,
                                   None, None, None, None, None, None, None, None, *map(ptr, out), ptr(w), w.nbytes,
                                   None), "vd_sw_step_tgl")
        return out

    def adj(self, x, a, nstep):
        B = x[0].shape[0]
        x, a = [self.c(t) for t in x], [self.c(t) for t in a]
        out = [np.empty(s, self.dtype) for s in self.shapes(B)]
        w = self.ws(B, nstep)
        ok(self.lib.vd_sw_step_adj(self.h, B, *map(ptr, x), *map(ptr, a), nstep, None, None, None, None, None, None,
                                   None, None, *map(ptr, out), None, None, None, None, None, None, ptr(w), w.nbytes,
                                   None), "vd_sw_step_adj")
        return out


def neumann(lib, nx, ny, dx, dy, lam, dtype):
    keep = [np.ascontiguousarray(np.asarray(a, dtype=np.float64)) for a in (dx, dy, lam)]
    h = ctypes.c_void_p()
    ok(lib.vd_neumann_plan_create(ctypes.byref(h), nx, ny, _lib.VD_F64 if dtype == np.float64 else _lib.VD_F32,
                                  ptr(keep[0]), ptr(keep[1]), int(keep[0].size > 1), ptr(keep[2]),
                                  int(keep[2].size > 1)), "vd_neumann_plan_create")
    return h


def helm_of(nx, ny, dx, dy, lam):
    x, y = np.meshgrid(np.arange(nx, dtype=np.float64), np.arange(ny, dtype=np.float64), indexing="ij")
    return 2 * (np.cos(np.pi / nx * x) - 1) / dx ** 2 + 2 * (np.cos(np.pi / ny * y) - 1) / dy ** 2 - lam


def ref_solve(rhs, helm):
    return SWOracle.neumann_solve(types.SimpleNamespace(helm_dct=helm), rhs)


# ---------------------------------------------------------------- the solve
@pytest.mark.parametrize("nx,ny,nf", [(8, 6, 1), (12, 10, 3), (14, 22, 2), (9, 15, 3), (6, 30, 1), (26, 39, 2),
                                      (64, 48, 1), (11, 13, 2), (8, 6, 400), (12, 10, 161)])
def test_neumann_solve(emu, nx, ny, nf):
    """Radix 4/2/3/5 and direct (7, 11, 13) stages, odd lengths, an odd
    number of rows and of columns (the paired transforms' padding); the large
    batches run 2 row pairs and 4 column pairs per CTA (small ones 1 and 1)."""
    rng = np.random.default_rng(nx * 100 + ny)
    dx = 1e4 * (1 + 0.2 * rng.random((nx, ny)))
    dy = 1.3e4 * (1 + 0.2 * rng.random((nx, ny)))
    lam = 1e-9 * (1 + rng.random((nx, ny)))
    helm = helm_of(nx, ny, dx, dy, lam)
    rhs = rng.standard_normal((nf, nx, ny))
    want = ref_solve(rhs, helm)
    for dt, tol in ((np.float64, 1e-12), (np.float32, 2e-5)):
        h = neumann(emu, nx, ny, dx, dy, lam, dt)
        try:
            r = np.array(rhs, dtype=dt)
            out = np.empty_like(r)
            ok(emu.vd_neumann_solve(h, nf, ptr(r), ptr(out), None), "vd_neumann_solve")
            assert rel(out, want) < tol, (dt, rel(out, want))
            ok(emu.vd_neumann_solve(h, nf, ptr(r), ptr(r), None), "in place")
            assert np.array_equal(r, out)
        finally:
            emu.vd_neumann_plan_destroy(h)


def test_neumann_golden(emu, g):
    """The reference's own solver's eigenvalues and solve (float64)."""
    nx, ny = 24, 20
    H = g["fa_H"]
    lam = 1.0 / (g["fa_gp"][0] * 30.0 * 60.0 * H.sum())
    want_helm = g["fa_helm_dct"][0]
    assert rel(helm_of(nx, ny, g["fa_dx"], g["fa_dy"], lam), want_helm) < 1e-14
    h = neumann(emu, nx, ny, g["fa_dx"], g["fa_dy"], np.array([lam]), np.float64)
    try:
        r = np.ascontiguousarray(g["fa_rhs"].reshape(1, nx, ny))
        out = np.empty_like(r)
        ok(emu.vd_neumann_solve(h, 1, ptr(r), ptr(out), None), "vd_neumann_solve")
        assert rel(out, g["fa_sol"].reshape(1, nx, ny)) < 1e-12
    finally:
        emu.vd_neumann_plan_destroy(h)


def test_neumann_refusals(emu):
    h = ctypes.c_void_p()
    one = np.array([1.0])
    zero = np.array([0.0])
    assert emu.vd_neumann_plan_create(ctypes.byref(h), 8, 8, _lib.VD_F64, ptr(one), ptr(one), 0, ptr(zero), 0) == 1
    assert emu.vd_neumann_plan_create(ctypes.byref(h), 8000, 8, _lib.VD_F64, ptr(one), ptr(one), 0, ptr(one), 0) == 4
    assert emu.vd_neumann_plan_create(ctypes.byref(h), 1, 8, _lib.VD_F64, ptr(one), ptr(one), 0, ptr(one), 0) == 1


# ---------------------------------------------------------------- the model
def _gparam(g):
    p = "fa_"
    return dict(nx=24, ny=20, nl=2, dx=g[p + "dx"], dy=g[p + "dy"], H=g[p + "H"], g_prime=g[p + "gp"], f=g[p + "f"],
                taux=0.05, tauy=-0.03, bottom_drag_coef=1e-6, dt=30.0, slip_coef=0.5, visc_coef=10.0, diff_coef=5.0,
                barotropic_filter=True, barotropic_filter_spectral=True)


def test_rhs_and_steps_golden(emu, g):
    prm = _gparam(g)
    o = SWOracle(prm)
    pl = Plan(emu, prm)
    u, v, h = o.to_model(g["fa_u0"], g["fa_v0"], g["fa_h0"])
    du, dv, dh = pl.rhs(u, v, h)
    assert rel(du, g["fa_dtu"]) < 1e-12 and rel(dv, g["fa_dtv"]) < 1e-12 and rel(dh, g["fa_dth"]) < 1e-12
    r = pl.step(g["fa_u0"], g["fa_v0"], g["fa_h0"], 3)
    for a, k in zip(r, ["u3", "v3", "h3"]):
        assert rel(a, g["fa_" + k]) < 1e-12, k
    # float32 plan, same case
    r32 = Plan(emu, prm, dtype=np.float32).step(g["fa_u0"], g["fa_v0"], g["fa_h0"], 3)
    for a, k in zip(r32, ["u3", "v3", "h3"]):
        assert rel(a, g["fa_" + k]) < 2e-5, k


def _case(nx=14, ny=10, nl=3, B=2, seed=5):
    rng = np.random.default_rng(seed)
    dx = 2e3 * (1 + 0.15 * rng.random((nx, ny)))
    dy = 2.5e3 * (1 + 0.15 * rng.random((nx, ny)))
    f = 1e-4 + 2e-11 * np.arange(ny + 1)[None, :] * 2.5e3 + np.zeros((nx + 1, 1))
    H = np.array([150.0, 350.0, 800.0]).reshape(nl, 1, 1)
    prm = dict(nx=nx, ny=ny, nl=nl, dx=dx, dy=dy, H=H, g_prime=np.array([9.81, 0.02, 0.01]), f=f, taux=0.04,
               tauy=-0.02, bottom_drag_coef=2e-6, dt=20.0, slip_coef=0.7, visc_coef=5.0, diff_coef=2.0,
               barotropic_filter=True, barotropic_filter_spectral=True)
    o = SWOracle(prm)
    m = o.masks
    u0 = 0.05 * rng.standard_normal((B, nl, nx + 1, ny)) * m.u
    v0 = 0.05 * rng.standard_normal((B, nl, nx, ny + 1)) * m.v
    h0 = 0.4 * rng.standard_normal((B, nl, nx, ny))
    return prm, o, (u0, v0, h0), rng


def test_steps_vs_oracle(emu):
    """Non-uniform spacings (the filter's per-point eigenvalues), 3 layers,
    2 batch members."""
    prm, o, x, _ = _case()
    r = Plan(emu, prm).step(*x, 4)
    want = o.step(*x, nstep=4)
    for a, b, k in zip(r, want, "uvh"):
        assert rel(a, b) < 1e-11, k
    # the filter is not a no-op on this case
    off = Plan(emu, dict(prm, barotropic_filter=False)).step(*x, 4)
    assert rel(off[0], want[0]) > 1e-6


def test_tangent_and_adjoint(emu):
    prm, o, x, rng = _case()
    pl = Plan(emu, prm)
    m = o.masks
    dx = (0.01 * rng.standard_normal(x[0].shape) * m.u, 0.01 * rng.standard_normal(x[1].shape) * m.v,
          0.1 * rng.standard_normal(x[2].shape))
    n = 3
    tl = pl.tgl(x, dx, n)
    eps = 1e-5
    p = pl.step(*[a + eps * b for a, b in zip(x, dx)], n)
    q = pl.step(*[a - eps * b for a, b in zip(x, dx)], n)
    for t, a, b, k in zip(tl, p, q, "uvh"):
        fd = (a - b) / (2 * eps)
        assert rel(t, fd) < 1e-6, k
    a1 = [rng.standard_normal(s) for s in pl.shapes(2)]
    ad = pl.adj(x, a1, n)
    lhs = sum(np.vdot(t, a) for t, a in zip(tl, a1))
    rhs = sum(np.vdot(d, a) for d, a in zip(dx, ad))
    assert abs(lhs - rhs) / abs(lhs) < 1e-12


def test_tangent_and_adjoint_float32(emu):
    """The float32 plan: the tangent against the float64 tangent, the
    adjoint by a dot product in float64 sums."""
    prm, o, x, rng = _case()
    m = o.masks
    dx = (0.01 * rng.standard_normal(x[0].shape) * m.u, 0.01 * rng.standard_normal(x[1].shape) * m.v,
          0.1 * rng.standard_normal(x[2].shape))
    p32, p64 = Plan(emu, prm, dtype=np.float32), Plan(emu, prm)
    tl32, tl64 = p32.tgl(x, dx, 2), p64.tgl(x, dx, 2)
    for a, b, k in zip(tl32, tl64, "uvh"):
        assert rel(a, b) < 1e-3, k
    a1 = [rng.standard_normal(s) for s in p32.shapes(2)]
    ad = p32.adj(x, a1, 2)
    lhs = sum(np.vdot(t.astype(np.float64), a) for t, a in zip(tl32, a1))
    rhs = sum(np.vdot(d, a.astype(np.float64)) for d, a in zip(dx, ad))
    assert abs(lhs - rhs) / abs(lhs) < 1e-4


def test_H_cotangent(emu):
    """The adjoint's cotangent of H (through the face thicknesses of the
    filter as well as the rest of the step) against central differences of
    the forward in H, the filter's lambd staying the model's own."""
    prm, o, x, rng = _case(B=1)
    nx, ny, nl = prm["nx"], prm["ny"], prm["nl"]
    H0 = prm["H"]
    lam = 1.0 / (9.81 * prm["dt"] * 2 * prm["dt"] * H0.sum())
    Hs = np.broadcast_to(H0, (nl, nx, ny)).copy()
    pl = Plan(emu, dict(prm, H=Hs), bf_lambd=np.array([lam]))
    n = 2
    a1 = [rng.standard_normal(s) for s in pl.shapes(1)]
    buf = np.zeros(emu.vd_sw_ref_adj_bytes(pl.h) // 8)
    ok(emu.vd_sw_set_ref_adj(pl.h, ptr(buf)), "set_ref_adj")
    pl.adj(x, a1, n)
    ok(emu.vd_sw_set_ref_adj(pl.h, None), "unset")
    adH = np.zeros((nl, nx, ny))
    ok(emu.vd_sw_ref_pullback(pl.h, ptr(buf), ptr(adH), None, None), "pullback")
    dH = rng.standard_normal((nl, nx, ny))
    eps = 1e-3
    fp = Plan(emu, dict(prm, H=Hs + eps * dH), bf_lambd=np.array([lam]), H_wind=H0).step(*x, n)
    fm = Plan(emu, dict(prm, H=Hs - eps * dH), bf_lambd=np.array([lam]), H_wind=H0).step(*x, n)
    lhs = sum(np.vdot((a - b) / (2 * eps), c) for a, b, c in zip(fp, fm, a1))
    rhs = np.vdot(adH, dH)
    assert abs(lhs - rhs) / abs(lhs) < 1e-6
    # the same direction through the tangent with respect to H
    tb = np.zeros_like(buf)
    ok(emu.vd_sw_set_ref_tangent(pl.h, ptr(dH), None, ptr(tb)), "set_ref_tangent")
    tl = pl.tgl(x, [np.zeros_like(a) for a in x], n)
    ok(emu.vd_sw_set_ref_tangent(pl.h, None, None, None), "unset tangent")
    assert abs(sum(np.vdot(t, c) for t, c in zip(tl, a1)) - lhs) / abs(lhs) < 1e-6


def test_H_cotangent_per_layer(emu):
    """A model whose H has unit spatial axes: its cotangent is that of
    per-layer thicknesses (no reference pressure gradients, sw.py:403-404),
    checked with a direction constant in space against the tangent."""
    prm, o, x, rng = _case(B=2)
    nx, ny, nl = prm["nx"], prm["ny"], prm["nl"]
    pl = Plan(emu, prm)
    n = 2
    a1 = [rng.standard_normal(s) for s in pl.shapes(2)]
    buf = np.zeros(emu.vd_sw_ref_adj_bytes(pl.h) // 8)
    ok(emu.vd_sw_set_ref_adj(pl.h, ptr(buf)), "set_ref_adj")
    pl.adj(x, a1, n)
    ok(emu.vd_sw_set_ref_adj(pl.h, None), "unset")
    adH = np.zeros((nl, nx, ny))
    ok(emu.vd_sw_ref_pullback(pl.h, ptr(buf), ptr(adH), None, None), "pullback")
    dH = np.broadcast_to(rng.standard_normal((nl, 1, 1)), (nl, nx, ny)).copy()
    tb = np.zeros_like(buf)
    ok(emu.vd_sw_set_ref_tangent(pl.h, ptr(dH), None, ptr(tb)), "set_ref_tangent")
    tl = pl.tgl(x, [np.zeros_like(a) for a in x], n)
    ok(emu.vd_sw_set_ref_tangent(pl.h, None, None, None), "unset tangent")
    lhs = sum(np.vdot(t, c) for t, c in zip(tl, a1))
    assert abs(lhs - np.vdot(adH, dH)) / abs(lhs) < 1e-12


def test_land_refused(emu):
    prm, _, _, _ = _case()
    mask = np.ones((prm["nx"], prm["ny"]))
    mask[4:6, 3:5] = 0
    d = dict(prm, mask=mask)
    with pytest.raises(AssertionError, match="VD_ERR_UNSUPPORTED"):
        _plan_with_mask(emu, d)


def _plan_with_mask(lib, prm):
    keep = []

    def arr(a):
        a = np.ascontiguousarray(np.asarray(a, dtype=np.float64))
        keep.append(a)
        return a.ctypes.data_as(DP)

    d = _lib.VdSwDesc()
    nx, ny, nl = prm["nx"], prm["ny"], prm["nl"]
    d.nx, d.ny, d.nl, d.dtype = nx, ny, nl, _lib.VD_F64
    d.dx_host, d.dy_host, d.f_host = arr(prm["dx"]), arr(prm["dy"]), arr(prm["f"])
    d.H_host, d.g_prime_host, d.mask_host = arr(prm["H"].reshape(nl)), arr(prm["g_prime"]), arr(prm["mask"])
    d.dt, d.slip_coef = prm["dt"], 1.0
    d.barotropic_filter = 1
    h = ctypes.c_void_p()
    ok(lib.vd_sw_plan_create(ctypes.byref(h), ctypes.byref(d)), "vd_sw_plan_create")
    lib.vd_sw_plan_destroy(h)


# ---------------------------------------------------------------- without the filter
def test_unfiltered_model_golden(emu):
    """The right-hand side drivers shared with the filter, on the reference's
    outputs of the model without it (tests/golden/sw_golden.npz: land,
    sponge, forcing and wind arrays; mass-consistent forcing with a scalar
    mixed-layer depth and a spatial H)."""
    g = dict(np.load(os.path.join(HERE, "golden", "sw_golden.npz")))
    p = "swa_"
    pa = dict(nx=28, ny=22, nl=2, dx=g[p + "dx"], dy=g[p + "dy"], f=g[p + "f"], H=g[p + "H"], g_prime=g[p + "gp"],
              dt=15.0, mask=g[p + "mask"], slip_coef=0.5, bottom_drag_coef=2e-7, visc_coef=30.0, diff_coef=20.0,
              sponge_coef=0.3, taux=g[p + "taux0"], tauy=g[p + "tauy0"], sponge_u=g[p + "sponge_u"],
              sponge_v=g[p + "sponge_v"], sponge_h=g[p + "sponge_h"])
    pl = Plan(emu, pa)
    o = SWOracle(dict(pa, taux=g[p + "taux0"], tauy=g[p + "tauy0"]))
    u, v, h = o.to_model(g[p + "u0"], g[p + "v0"], g[p + "h0"])
    du, dv, dh = pl.rhs(u, v, h, taux=g[p + "taux"], tauy=g[p + "tauy"])
    assert rel(du, g[p + "dtu"]) < 1e-12 and rel(dv, g[p + "dtv"]) < 1e-12 and rel(dh, g[p + "dth"]) < 1e-12
    r = pl.step(*(g[p + k] for k in ("u0", "v0", "h0")), 4, *(g[p + k] for k in ("ub", "vb", "hb", "Fu", "Fv", "Fh",
                                                                                    "taux", "tauy")))
    for a, k in zip(r, ["u4", "v4", "h4"]):
        assert rel(a, g[p + k]) < 1e-12, k
    p = "swb_"
    pb = dict(nx=24, ny=26, nl=1, dx=g[p + "dx"], dy=g[p + "dy"], f=g[p + "f"], H=g[p + "H"], g_prime=g[p + "gp"],
              dt=60.0, slip_coef=1.0, bottom_drag_coef=1e-6, h_wind=80.0, forcing_momentum="mass_consistent",
              h_min=0.05, taux=0.0, tauy=0.0)
    r = Plan(emu, pb).step(*(g[p + k] for k in ("u0", "v0", "h0")), 5, Fu=np.zeros_like(g[p + "u0"]),
                           Fv=np.zeros_like(g[p + "v0"]), Fh=g[p + "Fh"], taux=g[p + "taux"], tauy=g[p + "tauy"])
    for a, k in zip(r, ["u5", "v5", "h5"]):
        assert rel(a, g[p + k]) < 1e-12, k


# ---------------------------------------------------------------- open boundaries
def _obc_param(g, **over):
    p = "ob_"
    d = dict(nx=28, ny=22, nl=2, dx=g[p + "dx"], dy=g[p + "dy"], H=g[p + "H"], g_prime=g[p + "gp"], f=g[p + "f"],
             taux=0.04, tauy=-0.02, bottom_drag_coef=1e-6, dt=20.0, mask=g[p + "mask"], slip_coef=0.6,
             visc_coef=20.0, diff_coef=10.0, sponge_coef=0.2, flag_obc=True, sponge_u=g[p + "sponge_u"],
             sponge_v=g[p + "sponge_v"], sponge_h=g[p + "sponge_h"])
    d.update(over)
    return d


def test_open_boundaries_golden(emu):
    g = dict(np.load(os.path.join(HERE, "golden", "swobc_golden.npz")))
    prm = _obc_param(g)
    pl = Plan(emu, prm)
    o = SWOracle(prm)
    u, v, h = o.to_model(g["ob_u0"], g["ob_v0"], g["ob_h0"])
    du, dv, dh = pl.rhs(u, v, h)
    assert rel(du, g["ob_dtu"]) < 1e-12 and rel(dv, g["ob_dtv"]) < 1e-12 and rel(dh, g["ob_dth"]) < 1e-12
    r = pl.step(*(g["ob_" + k] for k in ("u0", "v0", "h0")), 4,
                *(g["ob_" + k] for k in ("ub", "vb", "hb", "Fu", "Fv", "Fh")))
    for a, k in zip(r, ("u4", "v4", "h4")):
        assert rel(a, g["ob_" + k]) < 1e-12, k
    # the inflow velocities on the walls are kept, and relaxed by the sponge
    assert np.abs(r[0][:, :, 0]).max() > 0 and np.abs(r[1][:, :, :, -1]).max() > 0


def test_open_boundaries_adjoint(emu):
    g = dict(np.load(os.path.join(HERE, "golden", "swobc_golden.npz")))
    pl = Plan(emu, _obc_param(g))
    rng = np.random.default_rng(3)
    x = [g["ob_" + k] for k in ("u0", "v0", "h0")]
    dx = [0.01 * rng.standard_normal(a.shape) for a in x]
    tl = pl.tgl(x, dx, 2)
    eps = 1e-6
    p = pl.step(*[a + eps * b for a, b in zip(x, dx)], 2)
    q = pl.step(*[a - eps * b for a, b in zip(x, dx)], 2)
    for t, a, b in zip(tl, p, q):
        assert rel(t, (a - b) / (2 * eps)) < 1e-6
    a1 = [rng.standard_normal(a.shape) for a in tl]
    ad = pl.adj(x, a1, 2)
    lhs = sum(np.vdot(t, a) for t, a in zip(tl, a1))
    assert abs(lhs - sum(np.vdot(d, a) for d, a in zip(dx, ad))) / abs(lhs) < 1e-12


# ---------------------------------------------------------------- mass-consistent forcing
def test_mass_consistent_forcing_adjoint(emu):
    """The forcing adjoint's gather (no atomics) with land next to the faces
    it averages over: dot products of the step's tangent (state and forcing
    directions) against its adjoint (state and forcing cotangents)."""
    g = dict(np.load(os.path.join(HERE, "golden", "sw_golden.npz")))
    p = "swa_"
    prm = dict(nx=28, ny=22, nl=2, dx=g[p + "dx"], dy=g[p + "dy"], f=g[p + "f"], H=g[p + "H"], g_prime=g[p + "gp"],
               dt=15.0, mask=g[p + "mask"], slip_coef=0.5, bottom_drag_coef=2e-7, visc_coef=30.0, diff_coef=20.0,
               taux=0.03, tauy=-0.01, forcing_momentum="mass_consistent")
    pl = Plan(emu, prm)
    rng = np.random.default_rng(11)
    B, n = 2, 2
    shp = pl.shapes(B)
    c = pl.c
    x = [c(0.1 * rng.standard_normal(s)) for s in shp]
    F = [c(np.zeros(shp[0])), c(np.zeros(shp[1])), c(1e-4 * rng.standard_normal(shp[2]))]
    dx = [c(0.01 * rng.standard_normal(s)) for s in shp]
    dF = [c(np.zeros(shp[0])), c(np.zeros(shp[1])), c(1e-5 * rng.standard_normal(shp[2]))]
    tl = [np.empty(s) for s in shp]
    w = pl.ws(B, n)
    ok(emu.vd_sw_step_tgl(pl.h, B, *map(ptr, x), *map(ptr, dx), n, None, None, None, None, None, None,
                          *map(ptr, F), *map(ptr, dF), None, None, *map(ptr, tl), ptr(w), w.nbytes, None), "tgl")
    a1 = [c(rng.standard_normal(s)) for s in shp]
    ad = [np.empty(s) for s in shp]
    adF = [np.empty(s) for s in shp]
    w = pl.ws(B, n)
    ok(emu.vd_sw_step_adj(pl.h, B, *map(ptr, x), *map(ptr, a1), n, None, None, None, *map(ptr, F), None, None,
                          *map(ptr, ad), None, None, None, *map(ptr, adF), ptr(w), w.nbytes, None), "adj")
    lhs = sum(np.vdot(t, a) for t, a in zip(tl, a1))
    rhs = sum(np.vdot(d, a) for d, a in zip(dx, ad)) + sum(np.vdot(d, a) for d, a in zip(dF, adF))
    assert abs(lhs - rhs) / abs(lhs) < 1e-12
    # the forcing's own cotangent is exercised (nonzero on ocean cells)
    assert np.abs(adF[2]).max() > 0
