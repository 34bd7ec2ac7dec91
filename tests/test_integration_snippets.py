"""The MEX gateway sources of the integration guide (its C code blocks)
compile (C99, -Wall -Wextra as errors) against include/bfe_gb300.h and a
stand-in mex.h: every call into the C ABI matches the declared signatures.
MATLAB itself is not needed and nothing is linked or run."""
import os
import re
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _blocks():
    text = open(os.path.join(ROOT, "INTEGRATION.md")).read()
    return re.findall(r"```c\n(.*?)```", text, flags=re.S)


def test_integration_has_the_gateway_sources():
    b = _blocks()
    assert len(b) >= 3
    assert "mexFunction" in b[0] and "bfe_plan_create_ex" in b[0] and "bfe_run(" in b[0]


@pytest.mark.parametrize("k", [0, 1, 2])
def test_gateway_block_compiles_against_the_abi(tmp_path, k):
    if shutil.which("gcc") is None:
        pytest.skip("no gcc")
    b = _blocks()
    helpers = b[0][:b[0].index("void mexFunction(")]
    src = b[0] if k == 0 else helpers + b[k]          # blocks 1, 2 reuse block 0's helpers
    f = tmp_path / ("gateway%d.c" % k)
    f.write_text(src)
    r = subprocess.run(["gcc", "-std=c99", "-Wall", "-Wextra", "-Werror", "-Wno-unused-parameter",
                        "-Wno-unused-function", "-fsyntax-only", "-I", os.path.join(ROOT, "tests", "mexstub"),
                        "-I", os.path.join(ROOT, "include"), str(f)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
