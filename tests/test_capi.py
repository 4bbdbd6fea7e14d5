"""CPU tests of the C ABI boundary: every declared symbol is exported with a
known signature, and host-side validation rejects bad systems before any
device work (the reference stops the process instead: get_irs.f90:30-38)."""
import ctypes as ct
import os
import re

import numpy as np
import pytest

import opaw_tddft_gb300 as pkg
from opaw_tddft_gb300 import synthetic

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "opaw_gb300.h")


def declared():
    txt = open(HEADER).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(opaw_[a-z0-9_]+)\s*\(", txt)))


def test_header_declares_the_path():
    names = declared()
    for must in ["opaw_dev_init", "opaw_h_apply_dev", "opaw_sn_apply_dev", "opaw_shs_apply_dev", "opaw_proj_dev",
                 "opaw_rhoij", "opaw_density", "opaw_nhat", "opaw_vks", "opaw_dij", "opaw_rebuild", "opaw_vh",
                 "opaw_excite", "opaw_dipole", "opaw_tddft_steps"]:
        assert must in names


def test_library_exports_every_declared_symbol():
    L = pkg.lib()
    for name in declared():
        assert hasattr(L, name), name
        assert name in pkg.SIGNATURES, name


def _ctx_status(s):
    st = pkg.Context.__new__(pkg.Context)
    try:
        pkg.Context.__init__(st, s)
    except pkg.OpawError as e:
        return e.status, str(e)
    st.close()
    return 0, ""


def test_box_outside_nonperiodic_grid_is_rejected():
    s = synthetic.small_system("tiny", norb=2)
    s.ir_start = s.ir_start.copy()
    s.ir_start[0, 0] = s.nx - 2  # box runs past the face
    status, msg = _ctx_status(s)
    assert status == 4 and "local grid cannot go outside box" in msg


def test_bad_grid_factor_is_rejected():
    s = synthetic.small_system("tiny", norb=2)
    s.nx = 34  # 2 * 17
    status, msg = _ctx_status(s)
    assert status == 1 and "prime factor" in msg


def test_bad_projector_count_is_rejected():
    s = synthetic.small_system("tiny", norb=2)
    s.ms = s.ms.copy()
    s.ms[0] = 17
    status, _ = _ctx_status(s)
    assert status == 1


def test_sphere_point_outside_grid_is_rejected():
    s = synthetic.small_system("tiny", norb=2)
    s.local_grid = s.local_grid.copy()
    s.local_grid[0, 2] = s.nz + 1
    status, _ = _ctx_status(s)
    assert status == 1


def test_null_arguments():
    L = pkg.lib()
    h = ct.c_void_p()
    assert L.opaw_dev_init(None, ct.byref(h)) == 1
    assert L.opaw_h_apply_dev(None, 0, 0, None, None, 1) == 1
    assert L.opaw_sync(None) == 1
    assert L.opaw_rconv(0, 1, 1, None, None, None) == 1


def test_no_device_reports_nodev():
    try:
        import torch

        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    s = synthetic.small_system("tiny", norb=2)
    status, msg = _ctx_status(s)
    assert status == 7 and "no CUDA device" in msg


def test_build_recipe_targets_sm103a():
    import importlib.util

    spec = importlib.util.spec_from_file_location("b", os.path.join(ROOT, "opaw-tddft_gb300", "build.py"))
    b = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(b)
    assert b.ARCH == ["-gencode", "arch=compute_103a,code=sm_103a"]
