"""The tensor-core (tcgen05, 3xTF32) x-direction DST-I pass against the
CUDA-core FMA pass and against the float64 oracle, on grids that exercise one
and several output tiles, odd transform lengths and ragged row tiles."""
import ctypes

import numpy as np
import pytest
import scipy.fft
import torch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def built():
    from vardyn_gb300 import build
    build.build()


def device_error():
    from vardyn_gb300 import _lib
    flag = ctypes.c_int(0)
    _lib.call("vd_device_error", ctypes.byref(flag), 1)
    return flag.value


def plan(n_y, n_x, engine):
    from vardyn_gb300.qg1l import QG1LPlan
    return QG1LPlan(n_y, n_x, 5e3, 5e3, 900.0, 1e-4, 2.7, time_scheme="rk2",
                    dtype=torch.float32, dst_engine=engine)


def dst_rows(p, field):
    """Spectral rows of the x-DST of the interior (parity-split order)."""
    from vardyn_gb300 import _lib
    B = field.shape[0]
    nbytes = _lib.load().vd_qg1l_spec_bytes(p.handle, B)
    spec = torch.zeros(nbytes // 4, dtype=torch.float32, device="cuda")
    st = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    _lib.call("vd_qg1l_dst_x", p.handle, B, ctypes.c_void_p(field.data_ptr()),
              ctypes.c_void_p(spec.data_ptr()), 0, None, st)
    torch.cuda.synchronize()
    return spec


def oracle_rows(field, ny, nx):
    """float64 DST-I of the interior rows, reordered even-k first then odd-k."""
    n = nx - 2
    y = scipy.fft.dst(field[:, 1:-1, 1:-1].astype(np.float64), type=1, norm="ortho", axis=-1)
    return np.concatenate([y[..., 0::2], y[..., 1::2]], axis=-1)


@pytest.mark.parametrize("ny,nx,B", [(64, 64, 1), (40, 66, 3), (130, 200, 2), (512, 512, 2), (300, 777, 1),
                                     (1024, 1024, 1)])
def test_tc_forward_pass_matches_oracle(ny, nx, B):
    rng = np.random.default_rng(ny + nx)
    f = rng.standard_normal((B, ny, nx)).astype(np.float32)
    ptc = plan(ny, nx, "auto")
    spec = dst_rows(ptc, torch.as_tensor(f, device="cuda"))
    assert device_error() == 0
    n = nx - 2
    lds = ((n + 3) // 4) * 4
    got = spec.view(B * (ny - 2), lds)[:, :n].cpu().numpy().reshape(B, ny - 2, n)
    exp = oracle_rows(f, ny, nx)
    err = np.linalg.norm(got - exp) / np.linalg.norm(exp)
    print(f"tc forward DST {ny}x{nx} B={B}: rel-L2 {err:.2e}")
    # 3xTF32 with fp32 accumulation: ~1e-7 * sqrt(transform length)
    assert err < 4e-6


@pytest.mark.parametrize("ny,nx,B", [(64, 64, 1), (130, 200, 2), (512, 512, 4), (300, 777, 1), (1024, 1024, 1)])
def test_tc_solve_matches_fma_and_oracle(ny, nx, B):
    from oracle.qg1l import QgmOracle
    rng = np.random.default_rng(3 * ny + nx)
    q = rng.standard_normal((B, ny, nx)) * 1e-6
    hb = rng.standard_normal((B, ny, nx)) * 1e-2
    qb = rng.standard_normal((B, ny, nx)) * 1e-7
    ptc, pfma = plan(ny, nx, "auto"), plan(ny, nx, "fma")
    args = [torch.as_tensor(a, dtype=torch.float32, device="cuda") for a in (q, hb, qb)]
    htc = ptc.pv2h(*args).cpu().numpy()
    hfma = pfma.pv2h(*args).cpu().numpy()
    assert device_error() == 0
    dx = np.full((ny, nx), 5e3)
    ref = QgmOracle(dx=dx, dy=dx, dt=900.0, c=2.7, f=1e-4, time_scheme="rk2")
    for b in range(B):
        exp = ref.pv2h(q[b], hb[b], qb[b])
        e_tc = np.linalg.norm(htc[b] - exp) / np.linalg.norm(exp)
        e_fma = np.linalg.norm(hfma[b] - exp) / np.linalg.norm(exp)
        print(f"solve {ny}x{nx}: tc {e_tc:.2e}  fma {e_fma:.2e}")
        assert e_tc < 3e-6 and e_fma < 3e-6


def test_tc_adjoint_epilogue_and_step():
    """Full model step and adjoint with the tensor-core solve (float32) against
    the same plan on CUDA-core FMA."""
    from vardyn_gb300.model_qg1l.jqgm import Qgm
    n = 96
    rng = np.random.default_rng(5)
    dx = np.full((n, n), 5e3)
    from vardyn_gb300.synthetic import kminus3_ssh
    h0 = kminus3_ssh(n, n, 5e3, 5e3, rng).astype(np.float32)
    hb = np.zeros((n, n), np.float32)
    m = Qgm(dx=dx, dy=dx, dt=900.0, c=2.7, f=1e-4, time_scheme="rk2", dtype="float32")
    ad = rng.standard_normal((n, n)).astype(np.float32)
    out_tc = m.step(h0, hb, 10)
    adj_tc = m.step_adj(ad, h0, hb, 10)
    from vardyn_gb300.qg1l import QG1LPlan
    pf = QG1LPlan(n, n, 5e3, 5e3, 900.0, 1e-4, 2.7, time_scheme="rk2", dtype=torch.float32,
                  dst_engine="fma", mask=m.mask)
    H0 = torch.as_tensor(h0, device="cuda")[None]
    HB = torch.as_tensor(hb, device="cuda")[None]
    out_f = pf.step(H0, HB, 10)[0].cpu().numpy()
    adj_f = pf.step_adj(torch.as_tensor(ad, device="cuda")[None], H0, HB, 10)[0].cpu().numpy()
    assert device_error() == 0
    assert np.linalg.norm(out_tc - out_f) / np.linalg.norm(out_f) < 2e-6
    assert np.linalg.norm(adj_tc - adj_f) / np.linalg.norm(adj_f) < 2e-5


@pytest.mark.parametrize("ny,nx,dtype,tol,B", [(40, 66, torch.float64, 1e-12, 2), (514, 512, torch.float32, 2e-6, 2),
                                              (130, 201, torch.float32, 2e-6, 2),
                                              (1024, 1024, torch.float32, 2e-6, 1),
                                              (1024, 1024, torch.float32, 2e-6, 2),
                                              (300, 500, torch.float64, 1e-12, 1),
                                              (1500, 260, torch.float32, 2e-6, 1)])
def test_tridiagonal_y_solve_matches_banded_solver(ny, nx, dtype, tol, B):
    """vd_qg1l_tridiag_y against scipy's banded solver on the same systems
    (column groups of 8, 16 and 32 per CTA, pieces of 32 and 64 rows)."""
    import scipy.linalg
    from vardyn_gb300 import _lib
    from vardyn_gb300.qg1l import QG1LPlan
    dx, dy, g, f, c = 5e3, 4e3, 9.81, 1e-4, 2.7
    p = QG1LPlan(ny, nx, dx, dy, 900.0, f, c, g=g, dtype=dtype)
    n, my = nx - 2, ny - 2
    ne = n - n // 2
    lds = ((n + 3) // 4) * 4
    rng = np.random.default_rng(ny)
    F = rng.standard_normal((B, my, lds))
    spec = torch.as_tensor(F, dtype=dtype, device="cuda").contiguous()
    st = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    _lib.call("vd_qg1l_tridiag_y", p.handle, B, ctypes.c_void_p(spec.data_ptr()), st)
    got = spec.cpu().numpy()
    a = g / f / dy ** 2
    for col in range(n):
        k = 2 * col if col < ne else 2 * (col - ne) + 1
        mu = 2 * (np.cos(np.pi / (nx - 1) * (k + 1)) - 1) / dx ** 2
        bk = g / f * (-2 / dy ** 2 + mu) - g * f / c ** 2
        ab = np.zeros((3, my))
        ab[0, 1:] = a
        ab[1, :] = bk
        ab[2, :-1] = a
        for b in range(B):
            x = scipy.linalg.solve_banded((1, 1), ab, F[b, :, col])
            err = np.linalg.norm(got[b, :, col] - x) / np.linalg.norm(x)
            assert err < tol, (col, err)
