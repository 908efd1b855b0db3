"""Host logic of the drop-in SW / QG classes (no GPU): the keyword sets they
build for their plans are accepted by the plan constructors (SWPlan, QGPlan),
with the barotropic filter and open boundaries on and off."""
import inspect

import numpy as np
import pytest
import torch

import vardyn_gb300.model_qgsw.qg as qgmod
import vardyn_gb300.model_qgsw.sw as swmod
from vardyn_gb300.qg_ml import QGPlan
from vardyn_gb300.sw import SWPlan


def _bare(cls, **param):
    """An instance with the attributes _plan_kwargs / _make_plan read."""
    nx, ny, nl = 8, 6, 2
    p = dict(nx=nx, ny=ny, nl=nl, dx=1e3, dy=1e3, f=np.full((nx + 1, ny + 1), 1e-4),
             H=np.array([100.0, 400.0]).reshape(2, 1, 1), g_prime=np.array([9.81, 0.02]), dt=10.0, taux=0.0,
             tauy=0.0)
    p.update(param)
    o = object.__new__(cls)
    o.param, o.nx, o.ny, o.nl = p, nx, ny, nl
    o.dtype = torch.float64
    o.H = p["H"]
    o._sponge = {"u": None, "v": None, "h": None}
    o.barotropic_filter = bool(p.get("barotropic_filter")) and cls is swmod.SW
    o.lambd = np.ones((1, 1, 1))
    return o


def _binder(real):
    sig = inspect.signature(real.__init__)

    def fake(*args, **kw):
        sig.bind(None, *args, **kw)   # TypeError on a keyword the plan does not take
        return kw
    return fake


@pytest.mark.parametrize("extra", [{}, {"barotropic_filter": True, "barotropic_filter_spectral": True},
                                   {"flag_obc": True}])
def test_sw_plan_keywords(monkeypatch, extra):
    monkeypatch.setattr(swmod.SW, "_plan_cls", staticmethod(_binder(SWPlan)))
    kw = _bare(swmod.SW, **extra)._make_plan(None)
    assert kw["barotropic_filter"] == bool(extra.get("barotropic_filter"))
    assert kw["flag_obc"] == bool(extra.get("flag_obc"))


@pytest.mark.parametrize("extra", [{}, {"barotropic_filter": True, "barotropic_filter_spectral": True}])
def test_qg_plan_keywords(monkeypatch, extra):
    monkeypatch.setattr(qgmod, "QGPlan", _binder(QGPlan))
    kw = _bare(qgmod.QG, **extra)._make_plan(None)
    assert "barotropic_filter" not in kw and "flag_obc" not in kw


def test_qg_open_boundaries_refused(monkeypatch):
    monkeypatch.setattr(qgmod, "QGPlan", _binder(QGPlan))
    with pytest.raises(NotImplementedError):
        _bare(qgmod.QG, flag_obc=True)._make_plan(None)
