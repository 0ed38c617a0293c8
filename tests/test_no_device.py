"""Without a CUDA device the library fails loudly: the calls that would
touch the GPU return null and report why (printed and through
pglGetLastError), and nothing falls back to the CPU.  Runs in a child
process with no visible device, so it behaves the same with or without a
GPU in the machine."""

import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CHILD = r"""
import ctypes, json
import numpy as np
import openpgl_gb300 as pgl
lib = pgl.load()
out = {}
dev = lib.pglNewDevice(pgl.PGL_DEVICE_TYPE_CPU_8, 0)
out["device"] = dev
out["device_error"] = pgl.last_error()
st = lib.pglNewSampleStorage()
out["storage"] = st
out["storage_error"] = pgl.last_error()
try:
    pgl.Device()
    out["raised"] = ""
except RuntimeError as e:
    out["raised"] = str(e)
print("RESULT " + json.dumps(out))
"""


def test_calls_fail_with_a_message_and_no_fallback():
    env = dict(os.environ, CUDA_VISIBLE_DEVICES="")
    p = subprocess.run([sys.executable, "-c", CHILD], cwd=ROOT, env=env, capture_output=True, text=True,
                       timeout=300)
    assert p.returncode == 0, p.stderr
    line = [l for l in p.stdout.splitlines() if l.startswith("RESULT ")][-1]
    r = json.loads(line[len("RESULT "):])
    assert r["device"] is None and r["storage"] is None
    assert r["device_error"].startswith("pglNewDevice: ") and len(r["device_error"]) > len("pglNewDevice: ")
    assert r["storage_error"].startswith("pglNewSampleStorage: ")
    assert r["raised"].startswith("pglNewDevice failed: ")
    # the message is also printed, as the reference's catch blocks print theirs
    assert "pglNewDevice: " in p.stdout
