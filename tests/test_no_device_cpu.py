"""Without a usable CUDA device the library fails loudly: initialisation and
every tensor operation raise XgbError; nothing falls back to a host path.
Runs in a child process (the library initialises once per process) and is
skipped where a device is present."""
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CHILD = r'''
import xped_gb300 as x
from xped_gb300 import Basis, Tensor
from xped_gb300._lib import XgbError
try:
    x.ensure_device(0)
    print("INIT-OK")
    raise SystemExit(0)
except XgbError as e:
    print("INIT-ERROR", e)
try:
    b = Basis.from_pairs("U1", [(-1, 1), (1, 1)])
    Tensor.zeros([b, b], [b, b])
    print("OP-OK")
except XgbError as e:
    print("OP-ERROR", e)
'''


def test_operations_raise_without_a_device():
    r = subprocess.run([sys.executable, "-c", CHILD], cwd=ROOT, capture_output=True, text=True, timeout=600)
    out = r.stdout
    if "INIT-OK" in out:
        pytest.skip("a CUDA device is present")
    assert r.returncode == 0, r.stderr
    assert "INIT-ERROR" in out
    assert "OP-ERROR" in out and "OP-OK" not in out
