"""Builds the CUDA library libwf.so (sm_103a) in-tree.

Each .cu translation unit is compiled in parallel, then linked with nvcc into
wavefrontpathtracing_gb300/_lib/libwf.so.  build(checked=True) makes the
bounds-checked variant _lib/libwf_checked.so (-DWF_CHECKED=1: every index a
kernel reads is checked before use; see csrc/wf_device.cuh), which the tests
run the GPU parity suite against a second time.  Device code is compiled with
--fmad=false and IEEE division / square root: the kernels' float results are
specified operation by operation (see csrc/wf_device.cuh), and the host side
(-ffp-contract=off) computes instance boxes and the emitter table the same way.
"""
import concurrent.futures
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIBDIR = os.path.join(HERE, "_lib")
LIB = os.path.join(LIBDIR, "libwf.so")
LIB_CHECKED = os.path.join(LIBDIR, "libwf_checked.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
SOURCES = ["wf_api.cu", "wf_trace.cu", "wf_shade.cu", "wf_tlas.cu", "wf_bvh.cu", "wf_batch.cu", "wf_mega.cu",
           "wf_sort.cu", "wf_qbvh.cu", "wf_texture.cu", "wf_image.cu"]


def nvcc():
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libwf.so")


def _flags():
    # WF_NVCC_DEFINES: extra -D tuning macros (for example -DWF_TRACE_MIN_BLOCKS=10); rebuild with force=True
    extra = os.environ.get("WF_NVCC_DEFINES", "").split()
    return ARCH + extra + ["-O3", "-lineinfo", "-std=c++17", "--fmad=false", "-prec-div=true", "-prec-sqrt=true",
                   "-Xcompiler", "-fPIC,-ffp-contract=off,-O2", "-Xptxas", "-warn-spills",
                   "-I", os.path.join(HERE, "..", "include")]


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose=False, force=False, checked=False):
    """Compiles libwf.so (or libwf_checked.so) if any source or header is newer
    than it; returns its path."""
    build_dir = BUILD + ("_checked" if checked else "")
    lib = LIB_CHECKED if checked else LIB
    defines = ["-DWF_CHECKED=1"] if checked else []
    os.makedirs(build_dir, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    headers += [os.path.join(HERE, "..", "include", f) for f in ("wf.h", "wf_shared.h")]
    cc = nvcc()
    jobs = []
    objs = []
    for src in SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(build_dir, src.replace(".cu", ".o"))
        objs.append(o)
        if force or _stale(o, [s] + headers):
            jobs.append([cc] + _flags() + defines + ["-c", s, "-o", o])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
        return r.stdout + r.stderr

    with concurrent.futures.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        for out in ex.map(run, jobs):
            if verbose and out.strip():
                print(out)
    if force or jobs or _stale(lib, objs):
        run([cc] + ARCH + ["-shared", "-o", lib] + objs)
    return lib


if __name__ == "__main__":
    print(build(verbose=True))
