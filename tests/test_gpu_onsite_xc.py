"""The on-site XC term of D_ij on the device (csrc/onsite_xc.cu) against the
oracle: the full D_ij of a rebuild, and the term alone as the difference of
two contexts that differ only in the radial tables."""
import dataclasses

import numpy as np
import pytest

import oracle as orc
import opaw_tddft_gb300 as pkg
from opaw_tddft_gb300 import synthetic

pytestmark = pytest.mark.gpu


def system(kind):
    if kind == "naphthalene":
        return synthetic.molecule("naphthalene")
    return synthetic.small_system(kind, norb=3)


@pytest.mark.parametrize("kind", ["tiny", "odd", "naphthalene"])
def test_dij_with_onsite_xc(kind):
    s = system(kind)
    psi = synthetic.orbitals(s, 3, seed=4).reshape(3, -1)
    s0 = dataclasses.replace(s, radial=None)
    o = orc.Oracle(s)
    d = {}
    for key, sy in (("xc", s), ("plain", s0)):
        c = pkg.Context(sy)
        c.set_vks(0, s.vks0)
        c.set_dij(0, s.dij_init)
        c.upload(0, psi)
        c.rebuild(0, pkg.PREC_FP64)
        d[key] = c.get_dij(0)
        rho = c.get_rhoij(0)
        c.close()
    o.set_vks(0, s.vks0)
    o.set_dij(0, s.dij_init)
    o.rebuild(psi, 0)
    ref = o.get_dij(0)
    assert np.abs(d["xc"] - ref).max() <= 1e-11 * np.abs(ref).max()
    dx = o.onsite_xc(rho)
    assert np.abs(dx).max() > 1e-3
    assert np.abs((d["xc"] - d["plain"]) - dx).max() <= 1e-11 * np.abs(ref).max()
