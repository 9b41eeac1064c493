"""The C-ABI library builds, loads without a GPU, and exports every entry point
include/qtip4pf_gb300.h declares (no compute calls are made here)."""
import ctypes
import os
import re

import pytest

from conftest import ROOT

HEADER = os.path.join(ROOT, "include", "qtip4pf_gb300.h")


def declared_symbols(path):
    text = open(path).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(qtg_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_entry_points():
    syms = declared_symbols(HEADER)
    for name in ("qtg_create", "qtg_neighbour_list", "qtg_get_forces", "qtg_kwald", "qtg_force_eval_sc",
                 "qtg_ftransform", "qtg_pile_g", "qtg_bussi", "qtg_get_kcv", "qtg_get_conserved", "qtg_update_class",
                 "qtg_update_pimd", "qtg_run_steps"):
        assert name in syms


def test_library_exports_every_declared_symbol():
    from qtip4pf_water_gb300 import build

    lib = ctypes.CDLL(build.build())
    missing = [s for s in declared_symbols(HEADER) if not hasattr(lib, s)]
    assert not missing, missing


def test_status_strings_without_gpu():
    import qtip4pf_water_gb300 as q

    L = q.load()
    assert L.qtg_status_string(0) == b"ok"
    assert L.qtg_status_string(3) == b"Verlet list overflow"


def test_create_rejects_bad_arguments_without_gpu():
    import qtip4pf_water_gb300 as q

    L = q.load()
    d = q.system_desc(64, 3, [20.0] * 3, propagator=q.SUZUKI_CHIN)  # odd P with Suzuki-Chin
    h = ctypes.c_void_p()
    arr = (q.SystemDesc * 1)(d)
    assert L.qtg_create(arr, 1, 0, ctypes.byref(h)) == 1
    d2 = q.system_desc(64, 4, [20.0] * 3)
    arr = (q.SystemDesc * 1)(d2)
    assert L.qtg_create(arr, 1, 7, ctypes.byref(h)) == 1  # bad precision


def test_python_mirror_raises_without_device():
    import qtip4pf_water_gb300 as q

    try:
        import torch

        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    with pytest.raises(q.QtgError):
        q.System.create(64, 4, [23.5] * 3)
