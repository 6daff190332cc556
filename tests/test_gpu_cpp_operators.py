"""The C++ operator layer (VExpand, HashJoin, Mintersect, TableConvert,
MatrixTableSelect, Count over the C ABI) runs the reference's own unit-test
cases and three query-plan shapes on the GPU (vertexsurge_gb300/cpp/vs_ops_test.cpp)."""
import subprocess

import pytest

from vertexsurge_gb300 import build

pytestmark = pytest.mark.gpu


def test_cpp_operator_suite():
    r = subprocess.run([str(build.OPS_TEST)], capture_output=True, text=True, timeout=600)
    print(r.stdout)
    print(r.stderr)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "0 failed" in r.stdout
