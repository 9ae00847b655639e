"""The reference-side binding documented in INTEGRATION.md compiles.

Section 1's ModelObjectGB300 (a ModelObject subclass that routes the hot path
through include/imfit_gb300.h) and section 2's mpfit side = 3 user function
are extracted from the document and compiled with g++ -fsyntax-only against
the reference's own headers (core/model_object.h:41-264,
function_objects/function_object.h:25-146) and this library's C header, so
the documented binding cannot drift from either interface: every `override`
must match a virtual of the reference's ModelObject and every imfit_* call
must match a declaration.  Skipped where the reference checkout is absent.
"""
import os
import re
import shutil
import subprocess

import pytest

import oracle

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _cpp_blocks(section_start, section_end):
    text = open(os.path.join(ROOT, "INTEGRATION.md")).read()
    sec = text[text.index(section_start):text.index(section_end)]
    return re.findall(r"```cpp\n(.*?)```", sec, re.S)


@pytest.mark.skipif(not oracle.reference_checkout() or shutil.which("g++") is None,
                    reason="reference checkout or g++ not present")
def test_documented_binding_compiles_against_reference_headers(tmp_path):
    cls = _cpp_blocks("## 1.", "## 2.")
    assert len(cls) == 1 and "class ModelObjectGB300 : public ModelObject" in cls[0]
    hook = [b for b in _cpp_blocks("## 2.", "## 3.") if "myfunc_mpfit_gb300" in b]
    assert len(hook) == 1
    (tmp_path / "model_object_gb300.h").write_text(cls[0])
    (tmp_path / "binding.cpp").write_text(
        '#include "model_object_gb300.h"\n#include <algorithm>\n#include <vector>\n\n' + hook[0] +
        "\nint use_binding() {\n  ModelObjectGB300 m(true, 0);\n  ModelObject *base = &m;\n"
        "  double p[3] = {0, 0, 0};\n  base->CreateModelImage(p);\n"
        "  return (int)base->GetFitStatistic(p) + myfunc_mpfit_gb300(1, 3, p, p, nullptr, base);\n}\n")
    ref = oracle.REFERENCE_DIR
    cmd = ["g++", "-std=c++17", "-fsyntax-only", "-Wall", "-Werror=overloaded-virtual", "-Werror=suggest-override",
           f"-I{tmp_path}", f"-I{ROOT}/include",
           # the reference's and the shims' headers as system headers: their own warnings are not checked
           "-isystem", f"{ref}/core", "-isystem", f"{ref}/function_objects", "-isystem", f"{ref}/solvers",
           "-isystem", ref, "-isystem", f"{ROOT}/oracle/shims", str(tmp_path / "binding.cpp")]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-4000:]
