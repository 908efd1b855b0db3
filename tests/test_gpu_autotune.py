"""The inversion schedule (vd_qg1l_set_schedule) and its autotuner
(vardyn_gb300.autotune): every schedule computes the same inversion, the
choices a plan cannot run are refused, the tuner sets its pick on the plan
and caches it."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def built():
    from vardyn_gb300 import build
    build.build()


def _plan(n, dtype):
    from vardyn_gb300.qg1l import QG1LPlan
    return QG1LPlan(n, n, 5e3, 5e3, 900.0, 1e-4, 2.7, time_scheme="rk2", dtype=dtype)


@pytest.mark.parametrize("n,dtype,tol", [(130, torch.float32, 2e-5), (130, torch.float64, 1e-12),
                                         (258, torch.float32, 2e-5)])
def test_every_schedule_gives_the_same_inversion(n, dtype, tol):
    from vardyn_gb300 import autotune
    p = _plan(n, dtype)
    rng = np.random.default_rng(1)
    q = torch.as_tensor(rng.standard_normal((3, n, n)) * 1e-5, dtype=dtype, device="cuda")
    hb = torch.as_tensor(rng.standard_normal((3, n, n)) * 1e-2, dtype=dtype, device="cuda")
    qb = p.h2pv(hb, hb)
    ref = p.pv2h(q, hb, qb).double()
    ran = 0
    for cand in autotune.candidates(p):
        p.set_schedule(**{k: 0 for k in p.SCHEDULE_KEYS})
        try:
            p.set_schedule(**cand)
        except RuntimeError:
            continue
        h = p.pv2h(q, hb, qb).double()
        err = float((h - ref).norm() / ref.norm())
        assert err <= tol, (cand, err)
        ran += 1
    # rule + (FMA rows [+ tensor-core groups]) x tridiagonal forms (8, 16, 32 rows [+ capped 16])
    assert ran >= (29 if dtype == torch.float32 else 7)


def test_refused_choices_and_tuner():
    from vardyn_gb300 import autotune
    p64 = _plan(130, torch.float64)
    with pytest.raises(RuntimeError):
        p64.set_schedule(engine=2)                # no tensor-core images for float64
    with pytest.raises(RuntimeError):
        p64.set_schedule(fma_rows=64)
    with pytest.raises(RuntimeError):
        p64.set_schedule(tridiag_rows=12)
    p = _plan(194, torch.float32)
    autotune.clear_cache()
    sched, times = autotune.tune(p, 4)
    assert len(times) >= 6
    cur = p.schedule()
    for k, v in sched.items():
        assert cur[k] == v
    best = min(times.values())
    assert best > 0
    p2 = _plan(194, torch.float32)
    s2, t2 = autotune.tune(p2, 4)                 # cached: same pick, set on the new plan
    assert s2 == sched and t2 is times
    assert all(p2.schedule()[k] == v for k, v in sched.items())
