"""The C-ABI library loads without a GPU and exports every symbol include/*.h declares."""
import ctypes
import glob
import os
import re

import pytest

import itk_gb300
from itk_gb300 import _capi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = []
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names += re.findall(r"^\s*(?:const\s+)?\w+\s*\*?\s*(gb_\w+)\s*\(", text, flags=re.M)
    return sorted(set(names))


def test_library_builds_and_loads():
    L = itk_gb300.lib()
    assert os.path.exists(itk_gb300.library_path())
    assert L.gb_version().decode().startswith("itk_gb300")


@pytest.mark.parametrize("name", declared_functions())
def test_symbol_exported(name):
    L = itk_gb300.lib()
    assert hasattr(L, name), f"{name} declared in include/ but not exported"
    assert name in _capi.SIGNATURES, f"{name} has no ctypes signature in itk_gb300/_capi.py"


def test_no_undeclared_signatures():
    declared = set(declared_functions())
    assert set(_capi.SIGNATURES) <= declared


def test_null_arguments_are_rejected_without_a_gpu():
    L = itk_gb300.lib()
    assert L.gb_metric_set_number_of_histogram_bins(None, 50) == _capi.GB_ERR_BAD_ARG
    assert "null" in _capi.last_error()
    assert L.gb_metric_initialize(None) == _capi.GB_ERR_BAD_ARG
    assert L.gb_ctx_create(0, None) == _capi.GB_ERR_BAD_ARG
    out = ctypes.c_void_p()
    rc = L.gb_ctx_create(0, ctypes.byref(out))
    # without a GPU the context cannot be created: a CUDA error, never a silent success
    assert rc in (_capi.GB_OK, _capi.GB_ERR_CUDA, _capi.GB_ERR_BAD_ARG)
    if rc == _capi.GB_OK:
        L.gb_ctx_destroy(out)
