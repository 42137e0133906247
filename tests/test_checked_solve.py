"""The acceptance rules of the drop-in layer's solve (models.checked_solve) on a fake solver: no GPU."""
import types

import numpy as np
import pytest
import torch

from opencmp_gb300 import _lib as LB
from opencmp_gb300.models import checked_solve


def _info(status, relres0, relres):
    i = LB.SolveInfo()
    i.status, i.relres0, i.relres = status, relres0, relres
    return i


class FakeSolver:
    """Returns the scripted infos in turn and records the initial guess of every call."""

    def __init__(self, infos, free):
        self.infos = list(infos)
        self.starts = []
        space = types.SimpleNamespace(FreeDofs=lambda: free)
        self.mat = types.SimpleNamespace(space=space)

    def solve(self, b, x, raise_on_fail=True):
        self.starts.append(x.clone())
        return self.infos.pop(0)


def test_accepts_converged_and_round_off_floor():
    free = np.ones(4, bool)
    for info in (_info(LB.OK, 1.0, 1e-13), _info(LB.NOT_CONVERGED, 1.0, 5e-10),
                 _info(LB.NOT_CONVERGED, 1e3, 5e-10 * 1e3 * 1e-3)):
        s = FakeSolver([info], free)
        assert checked_solve(s, torch.zeros(4), torch.ones(4), 1e-9) is info
        assert len(s.starts) == 1


def test_initial_residual_criterion():
    """NGSolve's criterion: a 1e-12 fall from the initial residual is accepted at the cap."""
    s = FakeSolver([_info(LB.NOT_CONVERGED, 1e10, 0.9e-2)], np.ones(3, bool))
    assert checked_solve(s, torch.zeros(3), torch.ones(3), 1e-9).relres == pytest.approx(0.9e-2)


def test_cancelled_rhs_retried_from_zero_on_free_dofs():
    """relres0 > 1 and no acceptance: the second solve starts from zero on the free dofs, the
    Dirichlet values stay."""
    free = np.array([True, False, True, True])
    x = torch.tensor([0.3, 7.0, 0.3, 0.3], dtype=torch.float64)
    s = FakeSolver([_info(LB.NOT_CONVERGED, 5e11, 0.9), _info(LB.OK, 1.0, 2e-13)], free)
    info = checked_solve(s, torch.zeros(4, dtype=torch.float64), x, 1e-9)
    assert info.status == LB.OK and len(s.starts) == 2
    assert torch.equal(s.starts[0], torch.tensor([0.3, 7.0, 0.3, 0.3], dtype=torch.float64))
    assert torch.equal(s.starts[1], torch.tensor([0.0, 7.0, 0.0, 0.0], dtype=torch.float64))


def test_no_retry_when_guess_was_better_than_zero():
    s = FakeSolver([_info(LB.NOT_CONVERGED, 0.5, 1e-3)], np.ones(2, bool))
    with pytest.raises(LB.OcmpError):
        checked_solve(s, torch.zeros(2), torch.ones(2), 1e-9)
    assert len(s.starts) == 1


def test_failed_retry_raises():
    s = FakeSolver([_info(LB.NOT_CONVERGED, 5e11, 0.9), _info(LB.NOT_CONVERGED, 1.0, 1e-3)], np.ones(2, bool))
    with pytest.raises(LB.OcmpError):
        checked_solve(s, torch.zeros(2), torch.ones(2), 1e-9)
    assert len(s.starts) == 2


def test_nonfinite_is_not_retried():
    s = FakeSolver([_info(LB.ERR_NONFINITE, float('nan'), float('nan'))], np.ones(2, bool))
    with pytest.raises(LB.OcmpError):
        checked_solve(s, torch.zeros(2), torch.ones(2), 1e-9)
