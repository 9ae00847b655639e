"""CPU checks of the C ABI: the library builds for sm_103a, loads without a
GPU, and exports exactly the entry points include/imfit_gb300.h declares.
No compute call is made here."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "imfit_gb300.h")


def declared_functions():
    txt = open(HEADER).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(imfit_\w+)\s*\(", txt)))


def test_header_declares_reference_entry_points():
    names = declared_functions()
    for must in ("imfit_SetupModelImage", "imfit_AddPSFVector", "imfit_AddImageDataVector",
                 "imfit_FinalSetupForFitting", "imfit_CreateModelImage", "imfit_ComputeDeviates",
                 "imfit_GetFitStatistic", "imfit_GetModelImageVector", "imfit_AddOversampledPsfInfo",
                 "imfit_UseCashStatistic", "imfit_UsePoissonMLR", "imfit_MakeBootstrapSample"):
        assert must in names


def test_library_builds_and_exports_every_declared_symbol(gpu):
    lib = ctypes.CDLL(gpu.library_path())
    for name in declared_functions():
        assert hasattr(lib, name), name
    # the Python mirror binds every declared symbol and nothing else
    assert sorted(gpu.exported_symbols()) == declared_functions()


def test_version_string(gpu):
    lib = gpu.load_library()
    assert b"sm_103a" in lib.imfit_Version()


def test_no_cpu_fallback_in_product_path():
    """The product package never imports the oracle."""
    pkg = os.path.join(ROOT, "imfit_gb300")
    for root, _, files in os.walk(pkg):
        for f in files:
            if f.endswith((".py", ".cpp", ".cu", ".cuh", ".h")):
                src = open(os.path.join(root, f)).read()
                assert "import oracle" not in src and "from oracle" not in src, f
                assert "liboracle" not in src and "imfit_oracle" not in src, f
