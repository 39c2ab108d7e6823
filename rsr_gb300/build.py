"""In-tree build of the GPU library and of the oracle's CPU libraries.

  rsr_gb300/librsrgpu.so     nvcc, sm_103a only, -fmad=false (the product)
  oracle/librsroracle.so     gcc, plain C restatement (test infrastructure)
  oracle/_ref/librsrref.so   rsr's own sources, x86-64 hosts with the
                             reference checkout only (test infrastructure)
"""
import os
import platform
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "librsrgpu.so")
ARCH = "-gencode=arch=compute_103a,code=sm_103a"
NVCC_FLAGS = [ARCH, "-O3", "-lineinfo", "-std=c++17", "-fmad=false", "-prec-div=true",
              "-prec-sqrt=true", "-ftz=false",
              "-Xcompiler", "-fPIC,-ffp-contract=off,-O2", "-I" + os.path.join(REPO, "include")]
SOURCES = ["rsrgpu_kernels.cu", "rsrgpu_host.cu", "rsrgpu_static.cu", "rsrgpu_deferred.cu", "rsrgpu_mlp.cu", "rsrgpu_learned.cu",
           "rsrgpu_texture.cu", "rsrgpu_postfx.cu", "rsrgpu_recorder.cu", "rsrgpu_perf.cu"]


def _reference_dir():
    """The reference checkout the oracle's reference build reads: $RSR_REFERENCE,
    else the default location the recipe oracle/ref/Makefile names."""
    if os.environ.get("RSR_REFERENCE"):
        return os.environ["RSR_REFERENCE"]
    r = subprocess.run(["make", "-s", "-C", os.path.join(REPO, "oracle", "ref"), "where"],
                       stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
    return r.stdout.strip() if r.returncode == 0 else ""


def _nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("command failed (%d): %s\n%s" % (r.returncode, " ".join(cmd), r.stdout))
    return r.stdout


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build_gpu(verbose=False, extra=()):
    os.makedirs(OBJ, exist_ok=True)
    nvcc = _nvcc()
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh", ".inc"))]
    headers.append(os.path.join(REPO, "include", "rsrgpu.h"))
    jobs = []
    objs = []
    for src in SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OBJ, src + ".o")
        objs.append(o)
        if _stale(o, [s] + headers + [__file__]):
            jobs.append([nvcc, *NVCC_FLAGS, *extra, "-c", s, "-o", o])
    with ThreadPoolExecutor(max_workers=len(jobs) or 1) as ex:
        for out in ex.map(_run, jobs):
            if verbose and out.strip():
                print(out)
    if _stale(LIB, objs):
        _run([nvcc, ARCH, "-shared", "-cudart", "static", "-o", LIB, *objs])
    return LIB


def build_oracle():
    src = os.path.join(REPO, "oracle", "rsr_oracle.c")
    out = os.path.join(REPO, "oracle", "librsroracle.so")
    deps = [src, os.path.join(REPO, "include", "rsrgpu.h"), os.path.join(CSRC, "rcpps_table.inc")]
    if _stale(out, deps):
        _run(["gcc", "-O2", "-std=c11", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared",
              "-pthread", "-o", out, src, "-lm"])
    return out


def build_reference():
    """Builds oracle/_ref when the reference checkout is present on an x86-64 host."""
    ref = _reference_dir()
    if not ref or not os.path.isdir(ref) or platform.machine() not in ("x86_64", "AMD64"):
        return None
    _run(["make", "-s", "-C", os.path.join(REPO, "oracle", "ref"), "-j8", "REF=" + ref])
    return os.path.join(REPO, "oracle", "_ref", "librsrref.so")


def build_shim_test():
    """Builds oracle/_ref/rsr_translate (include/rsrgpu_rglv.hpp against
    rsr's own headers and GL recorder) when the reference checkout is present
    on an x86-64 host; returns its path or None."""
    ref = _reference_dir()
    if not ref or not os.path.isdir(ref) or platform.machine() not in ("x86_64", "AMD64"):
        return None
    build_gpu()
    _run(["make", "-s", "-C", os.path.join(REPO, "oracle", "ref"), "-j8", "REF=" + ref, "shim"])
    return os.path.join(REPO, "oracle", "_ref", "rsr_translate")


def build_all(verbose=False):
    with ThreadPoolExecutor(max_workers=3) as ex:
        f_gpu = ex.submit(build_gpu, verbose)
        f_orc = ex.submit(build_oracle)
        f_ref = ex.submit(build_reference)
        return f_gpu.result(), f_orc.result(), f_ref.result()


if __name__ == "__main__":
    print(build_all(verbose="-v" in sys.argv))
