"""The autotuner's candidate schedules (host logic, no GPU): which inversion
forms it times for float32 and float64 plans, and that it leaves the adjoint
stage's staging field alone."""
import torch

from vardyn_gb300 import autotune


class FakePlan:
    SCHEDULE_KEYS = ("engine", "tc_group_fwd", "tc_group_inv", "fma_rows", "tridiag_rows", "tridiag_lean",
                     "stencil_loads")

    def __init__(self, dtype, dst_engine="auto"):
        self.dtype = dtype
        self.dst_engine = dst_engine


def test_float32_candidates():
    c = autotune.candidates(FakePlan(torch.float32))
    assert c[0] == {}                                        # the built-in rule first
    assert len(c) == 1 + (3 + 4) * 4                         # (FMA rows + TC groups) x tridiagonal forms
    assert {d.get("engine") for d in c[1:]} == {1, 2}
    assert {d.get("tridiag_rows") for d in c[1:]} == {8, 16, 32}
    assert any(d.get("tridiag_lean") == 1 for d in c)
    assert not any("stencil_loads" in d for d in c)


def test_float64_and_fma_only_candidates():
    c = autotune.candidates(FakePlan(torch.float64))
    assert len(c) == 1 + 2 * 3
    assert all(d.get("engine", 1) == 1 for d in c[1:])
    assert not any(d.get("tridiag_lean") for d in c)
    c = autotune.candidates(FakePlan(torch.float32, dst_engine="fma"))
    assert all(d.get("engine") == 1 for d in c[1:])


def test_tuner_resets_only_the_inversion_fields():
    keys = autotune._inv_keys(FakePlan(torch.float32))
    assert "stencil_loads" not in keys and "engine" in keys and "tridiag_rows" in keys
