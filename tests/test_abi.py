"""The C ABI library loads (no GPU needed) and exports every function include/wumingpic2d.h declares."""
import ctypes
import re
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
HEADER = ROOT / "include" / "wumingpic2d.h"


def declared_functions():
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(?:int|const char \*)\s*(wm_\w+)\s*\(", text)))


@pytest.fixture(scope="module")
def built_lib():
    from wumingpic2d_gb300 import build

    path = build.build()
    return ctypes.CDLL(str(path))


def test_header_declares_module_procedures():
    names = declared_functions()
    for n in ("wm_particle_init", "wm_particle_solv", "wm_field_init", "wm_field_fdtd_i", "wm_sort_init", "wm_sort_bucket",
              "wm_mom_calc_init", "wm_mom_calc_accl", "wm_mom_calc_nvt", "wm_bc_periodic_init", "wm_bc_periodic_particle_x",
              "wm_bc_periodic_particle_y", "wm_bc_periodic_dfield", "wm_bc_periodic_curre", "wm_bc_periodic_phi",
              "wm_bc_periodic_mom"):
        assert n in names


def test_every_declared_symbol_is_exported(built_lib):
    missing = [n for n in declared_functions() if not hasattr(built_lib, n)]
    assert not missing, missing


def test_python_binding_covers_header():
    from wumingpic2d_gb300._native import SIGNATURES

    assert set(declared_functions()) <= set(SIGNATURES)


def test_status_strings_without_gpu(built_lib):
    from wumingpic2d_gb300 import _native

    L = _native.lib()
    assert L.wm_status_string(0) == b"ok"
    assert b"sm_103a" in L.wm_build_info()


def test_api_rejects_c_ordered_arrays(built_lib):
    from wumingpic2d_gb300 import api

    a = np.zeros((6, 4, 4, 2))  # C order
    with pytest.raises(TypeError):
        api.particle__solv(a, a, a, np.zeros((5, 4, 2), dtype=np.int32, order="F"), 2, 5)


def test_api_init_rejects_bad_dimensions(built_lib):
    from wumingpic2d_gb300 import _native, api

    with pytest.raises(_native.WmError):
        api.particle__init(5, 10, 2, 2, 9, 2, 9, 2, 9, 1.0, 0.5, 1.0, [1.0, -1.0], [1.0, 1.0])  # ndim must be 6
    with pytest.raises(_native.WmError):
        api.sort__init(6, 10, 2, 2, 9, 2, 9, 3, 9)  # nys != nygs: one process owns every row
