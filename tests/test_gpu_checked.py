"""The GPU parity suite against the bounds-checked build.

libwf_checked.so is the same library compiled with WF_CHECKED: every index a
kernel reads from memory (node children, leaf triangles, instances, meshes,
hit primitives, textures, paths, queue slots, scene ids) is compared with the
size of what it indexes before the access, and a bad one raises
WF_ERR_BOUNDS from the next synchronising call.  This stands in for
compute-sanitizer, which this deployment cannot run: the render, traversal,
batch, texture, tail and megakernel parity tests run again in a child process
with WF_LIBRARY pointing at the checked build, and must pass unchanged (the
same images, hits and ray counts, and no bounds error)."""
import os
import subprocess
import sys

import pytest

from wavefrontpathtracing_gb300 import build as wfbuild

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SUITE = ["tests/test_gpu_render.py", "tests/test_gpu_trace.py", "tests/test_gpu_batch.py", "tests/test_gpu_qbvh.py",
         "tests/test_gpu_instance_bounds.py", "tests/test_gpu_textures.py", "tests/test_gltf.py", "tests/test_fbx.py"]


def test_checked_build_reports_itself():
    import ctypes
    lib = wfbuild.build(checked=True)
    L = ctypes.CDLL(lib)
    assert L.wf_checked_build() == 1
    assert ctypes.CDLL(wfbuild.build()).wf_checked_build() == 0


def test_parity_suite_under_bounds_checks():
    lib = wfbuild.build(checked=True)
    env = dict(os.environ, WF_LIBRARY=lib)
    code = ("import sys, pytest, wavefrontpathtracing_gb300 as wf\n"
            "assert wf.load().wf_checked_build() == 1\n"
            f"sys.exit(pytest.main({SUITE!r} + ['-m', 'gpu', '-x', '-q', '-p', 'no:cacheprovider']))\n")
    r = subprocess.run([sys.executable, "-c", code], cwd=ROOT, env=env, capture_output=True, text=True,
                       timeout=1500)
    assert r.returncode == 0, r.stdout[-4000:] + r.stderr[-2000:]
    assert " passed" in r.stdout
