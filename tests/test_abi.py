"""The C-ABI library builds, loads and exports every function include/lvgpu.h
declares (no GPU needed: nothing here launches a kernel)."""
import ctypes
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    src = open(os.path.join(ROOT, "include", "lvgpu.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(lv_[A-Za-z_0-9]+)\s*\(", src)))


def test_header_declares_the_api():
    names = declared_functions()
    for must in ("lv_create", "lv_remesh", "lv_move", "lv_find_pressure", "lv_pressure_step", "lv_relaxation_step",
                 "lv_export_system", "lv_destroy"):
        assert must in names


def test_library_exports_every_declared_symbol(lv):
    lib = ctypes.CDLL(lv._lib.LIB_PATH)
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_binding_covers_the_header(lv):
    assert set(declared_functions()) == set(lv._lib.SIGNATURES)


def test_create_without_gpu_fails_cleanly(lv):
    import torch
    if torch.cuda.is_available():
        return
    L = lv._lib.load()
    p = lv.LvParams()
    p.xmax[0] = p.xmax[1] = 1.0
    p.dr, p.capacity = 0.1, 10
    assert not L.lv_create(ctypes.byref(p))
