"""CPU: the C ABI library loads, exports every entry point include/*.h
declares, and reports errors (no GPU needed for any of this)."""
import ctypes
import os
import re

import numpy as np
import pytest

import wavefrontpathtracing_gb300 as wf
from wavefrontpathtracing_gb300 import abi, build

INCLUDE = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include")


def declared_symbols():
    names = set()
    for f in os.listdir(INCLUDE):
        if f.endswith(".h"):
            text = open(os.path.join(INCLUDE, f)).read()
            names |= set(re.findall(r"^\s*(?:const\s+)?\w+\**\s+\**(wf_\w+)\s*\(", text, flags=re.M))
    return names


@pytest.fixture(scope="module")
def lib():
    build.build()
    return wf.load()


def test_every_declared_symbol_is_exported_and_bound(lib):
    names = declared_symbols()
    assert len(names) >= 24
    assert names == set(wf.SIGNATURES), names ^ set(wf.SIGNATURES)
    for n in names:
        assert hasattr(lib, n), n


def test_status_strings_and_version(lib):
    assert lib.wf_abi_version() == 1
    assert lib.wf_status_string(0) == b"ok"
    assert lib.wf_status_string(-5) == b"traversal stack overflow"


def test_null_arguments_are_rejected_without_a_device(lib):
    h = ctypes.c_void_p()
    assert lib.wf_create(None, ctypes.byref(h)) == -1
    assert b"null" in lib.wf_last_error()
    assert lib.wf_destroy(None) == 0
    assert lib.wf_render(None, None, None, 0) == -1
    assert lib.wf_trace(None, None, 0, None, 0) == -1


def test_create_reports_missing_device_or_bad_size(lib):
    p = abi.InitParams(0, 16, 1, 0, 0, 0)
    h = ctypes.c_void_p()
    assert lib.wf_create(ctypes.byref(p), ctypes.byref(h)) == -1   # zero width
    p = abi.InitParams(16, 16, 1, 0, 0, 0)
    rc = lib.wf_create(ctypes.byref(p), ctypes.byref(h))
    if rc == 0:
        lib.wf_destroy(h)       # a GPU is present
    else:
        assert rc == -6 and b"device" in lib.wf_last_error()


def test_struct_layouts_match_the_reference_sizes():
    sizes = {"vertex": abi.vertex_dtype.itemsize, "triangle": abi.triangle_dtype.itemsize,
             "material": abi.material_dtype.itemsize, "ray": abi.ray_dtype.itemsize, "hit": abi.hit_dtype.itemsize,
             "bvh_instance": abi.bvh_instance_dtype.itemsize, "bvh_node": abi.bvh_node_dtype.itemsize,
             "tlas_node": abi.tlas_node_dtype.itemsize}
    assert sizes == {"vertex": 48, "triangle": 144, "material": 52, "ray": 32, "hit": 20, "bvh_instance": 92,
                     "bvh_node": 32, "tlas_node": 32}
    assert ctypes.sizeof(abi.View) == 272 and ctypes.sizeof(abi.RenderSettings) == 28


def test_product_does_not_import_the_oracle():
    pkg = os.path.dirname(wf.__file__)
    bad = re.compile(r"^\s*(from\s+oracle|import\s+oracle|#\s*include\s+.*oracle)|liborc|orc_\w+\(", re.M)
    for root, _, files in os.walk(pkg):
        for f in files:
            if f.endswith((".py", ".cu", ".h", ".cuh")):
                assert not bad.search(open(os.path.join(root, f)).read()), f


def test_ctypes_mirrors_match_the_c_header(tmp_path):
    """Every ctypes structure of the binding has the size and field offsets
    that a C compiler gives the include/wf.h declaration it mirrors."""
    import shutil
    import subprocess
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    pairs = {"RenderSettings": "render_settings_t", "View": "view_t", "InitParams": "wf_init_params",
             "BvhOptions": "wf_bvh_options", "Env": "wf_env", "RenderOptions": "wf_render_options",
             "Stats": "wf_stats", "BatchConfig": "wf_batch_config", "BatchStats": "wf_batch_stats"}
    lines = ["#include <stdio.h>", "#include <stddef.h>", '#include "wf.h"', "int main(void) {"]
    for py, c in pairs.items():
        lines.append('printf("%s size %%zu\\n", sizeof(%s));' % (py, c))
        for name, _ in getattr(abi, py)._fields_:
            lines.append('printf("%s %s %%zu\\n", offsetof(%s, %s));' % (py, name, c, name))
    lines.append("return 0; }")
    src = tmp_path / "sizes.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "sizes"
    inc = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include")
    subprocess.run([cc, "-std=c11", "-I", inc, str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split("\n")
    got = {}
    for line in out:
        if line:
            k, v = line.rsplit(" ", 1)
            got[k] = int(v)
    for py in pairs:
        cls = getattr(abi, py)
        assert got[py + " size"] == ctypes.sizeof(cls), py
        for name, _ in cls._fields_:
            assert got["%s %s" % (py, name)] == getattr(cls, name).offset, (py, name)
