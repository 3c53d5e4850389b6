"""The texture sampler's BC decode as a checker (tests/hw_sampler.cu, test
infrastructure): build() compiles it next to the library, decode() runs it."""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "hw_sampler.cu")
LIB = os.path.join(HERE, "_build", "libhw_sampler.so")
# wf_texture_create's BC formats -> the sampler's kinds (linear formats only:
# sRGB variants decode to the same bytes)
KINDS = {4: 1, 5: 1, 6: 2, 7: 2, 8: 3, 9: 3, 10: 4, 11: 5, 12: 7, 13: 7}
_lib = None


def build():
    from wavefrontpathtracing_gb300 import build as wfbuild
    if os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(SRC):
        return LIB
    os.makedirs(os.path.dirname(LIB), exist_ok=True)
    cmd = [wfbuild.nvcc()] + wfbuild.ARCH + ["-O2", "-shared", "-Xcompiler", "-fPIC", SRC, "-o", LIB]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return LIB


def lib():
    global _lib
    if _lib is None:
        _lib = ctypes.CDLL(build())
        _lib.hws_decode_bc.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint32,
                                       ctypes.c_void_p, ctypes.c_char_p, ctypes.c_int]
        _lib.hws_decode_bc.restype = ctypes.c_int
    return _lib


def decode(fmt, blocks, bw, bh):
    """bw x bh blocks of wf_texture_create format fmt -> (4 bh, 4 bw, 4)
    float32 texels as the sampler returns them (normalised, point-sampled)."""
    blocks = np.ascontiguousarray(blocks, dtype=np.uint8)
    out = np.zeros((4 * bh, 4 * bw, 4), np.float32)
    err = ctypes.create_string_buffer(256)
    rc = lib().hws_decode_bc(KINDS[fmt], blocks.ctypes.data, bw, bh, out.ctypes.data, err, 256)
    if rc != 0:
        raise RuntimeError("texture sampler decode failed: " + err.value.decode())
    return out
