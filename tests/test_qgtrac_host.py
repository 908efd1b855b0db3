"""Argument checks of the drop-in Qgm_trac that run before any device work."""
import numpy as np
import pytest

from vardyn_gb300.model_qg1l.jqgm import Qgm_trac

KW = dict(dx=np.full((12, 12), 1e4), dy=np.full((12, 12), 1e4), dt=900.0, SSH=np.zeros((12, 12)), c=2.7)


def test_unknown_time_scheme_is_refused():
    with pytest.raises(ValueError):
        Qgm_trac(time_scheme="rk3", **KW)


def test_ageostrophic_velocities_are_not_built():
    with pytest.raises(NotImplementedError):
        Qgm_trac(ageo_velocities=True, **KW)
