"""The product has no CPU path: without a CUDA device (or without libcctgpu.so) every
compute call raises, and nothing in the package imports the oracle."""
import os
import re
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "cctpy_gb300")

PROBE = r"""
import sys
import numpy as np
from cctpy_gb300 import (GPU_ACCELERATOR, HUST_SC_GANTRY, P3, ParticleFactory, ParticleRunner)

bl = HUST_SC_GANTRY().create_second_bending_part_beamline()   # placement is host geometry
calls = {
    "field": lambda: bl.magnetic_field_at(P3(0.1, 0.0, 0.0)),
    "field_points": lambda: bl.magnetic_field_at_points(np.zeros((4, 3)), "f32c"),
    "run_only": lambda: ParticleRunner.run_only(ParticleFactory.create_proton(P3(), P3(1, 0, 0)), bl, 0.01),
    "accelerator": lambda: GPU_ACCELERATOR().track_multi_particle_beamline_for_magnet_with_multi_qs(
        [bl], [ParticleFactory.create_proton(P3(), P3(1, 0, 0))], 0.01, 0.001),
}
for name, f in calls.items():
    try:
        f()
    except (RuntimeError, ImportError) as e:
        print(name, "raised", type(e).__name__)
    else:
        print(name, "COMPUTED")
print("oracle loaded" if any(m == "oracle" or m.startswith("oracle.") for m in sys.modules) else "oracle absent")
"""


def test_compute_calls_raise_without_a_device():
    env = dict(os.environ, CUDA_VISIBLE_DEVICES="")
    r = subprocess.run([sys.executable, "-c", PROBE], cwd=ROOT, env=env, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    out = r.stdout
    for name in ("field", "field_points", "run_only", "accelerator"):
        assert f"{name} raised" in out, out
    assert "COMPUTED" not in out
    assert "oracle absent" in out


def test_missing_library_raises():
    code = ("from cctpy_gb300 import _lib\n"
            "try:\n    _lib.load('/nonexistent/libcctgpu.so')\n"
            "except ImportError as e:\n    print('raised', 'build()' in str(e))\n")
    r = subprocess.run([sys.executable, "-c", code], cwd=ROOT, capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    assert r.stdout.strip() == "raised True"


def test_package_never_imports_the_oracle():
    pat = re.compile(r"^\s*(import\s+oracle|from\s+oracle[\s.])|['\"]oracle[/.]", re.M)
    for dirpath, _, files in os.walk(PKG):
        for f in files:
            if f.endswith((".py", ".cu", ".cuh", ".h")):
                text = open(os.path.join(dirpath, f), encoding="utf-8").read()
                assert not pat.search(text), os.path.join(dirpath, f)
