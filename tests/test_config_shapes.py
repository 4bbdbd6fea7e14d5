"""The synthetic systems of the configuration-shape GPU tests keep every
projector box inside the grid (the non-periodic rule of get_irs.f90:30-38,
which the device context enforces at set-up)."""
import numpy as np
import pytest

from opaw_tddft_gb300 import synthetic
from test_gpu_configs import SHAPES


@pytest.mark.parametrize("name", sorted(SHAPES))
def test_boxes_inside_grid(name):
    s = synthetic.build_system(norb=3, **SHAPES[name])
    ir = np.asarray(s.ir_start).reshape(-1, 3)  # 1-based
    nr = np.asarray(s.nrough).reshape(-1, 3)
    n = np.array([s.nx, s.ny, s.nz])
    assert (ir >= 1).all() and (ir + nr - 1 <= n).all()
    assert s.natom == SHAPES[name]["natom"]
