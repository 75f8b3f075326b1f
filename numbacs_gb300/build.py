"""Build ``numbacs_gb300/_build/libnbcs.so`` (sm_103a) from ``csrc/*.cu`` with nvcc.

Translation units are compiled in parallel and linked into one shared library
with a plain C ABI (``include/nbcs.h``).  The FP64 units that must reproduce the
reference arithmetic bit for bit are compiled with ``-fmad=false``; the mixed-
precision integrator is compiled with FMA contraction on.

    python -m numbacs_gb300.build          # build if sources changed
    python -m numbacs_gb300.build --force  # rebuild everything
    python -m numbacs_gb300.build --check  # the bounds-checked debug library,
                                           # _build_check/libnbcs_check.so (-DNBCS_CHECK)
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libnbcs.so")
BUILD_CHECK = os.path.join(HERE, "_build_check")
LIB_CHECK = os.path.join(BUILD_CHECK, "libnbcs_check.so")
INCLUDE = os.path.join(ROOT, "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-I", INCLUDE, "-I", CSRC,
          "--expt-relaxed-constexpr"]

# (source, extra flags)
SOURCES = [
    ("capi.cu", []),
    ("flowmap64.cu", ["-fmad=false"]),
    ("flowmap32.cu", []),
    ("ftle.cu", ["-fmad=false"]),
    ("spline.cu", ["-fmad=false"]),
    ("ridges.cu", ["-fmad=false"]),
    ("probe.cu", []),
    ("batch32.cu", []),
    ("batch64.cu", ["-fmad=false"]),
    ("mlp_train.cu", []),
    ("learned.cu", []),
    ("label.cu", []),
    ("compose.cu", ["-fmad=false"]),
    ("ordered.cu", ["-Xcompiler", "-ffp-contract=off"]),
]


def nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _deps():
    hdrs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    hdrs.append(os.path.join(INCLUDE, "nbcs.h"))
    return hdrs


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _compile(src, extra, verbose, bdir=BUILD):
    obj = os.path.join(bdir, src.replace(".cu", ".o"))
    cmd = [nvcc(), "-c", os.path.join(CSRC, src), "-o", obj] + ARCH + COMMON + extra
    if verbose:
        cmd += ["-Xptxas", "-v"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, " ".join(cmd), r.stderr))
    return obj, r.stderr


def build(force=False, verbose=False, jobs=None, check=False):
    """Compile every CUDA source for sm_103a and link libnbcs.so (with
    check=True: the bounds-checked libnbcs_check.so, -DNBCS_CHECK, in its own
    build folder). Returns its path."""
    bdir, lib = (BUILD_CHECK, LIB_CHECK) if check else (BUILD, LIB)
    flag = ["-DNBCS_CHECK"] if check else []
    os.makedirs(bdir, exist_ok=True)
    hdrs = _deps()
    todo = []
    for src, extra in SOURCES:
        obj = os.path.join(bdir, src.replace(".cu", ".o"))
        if force or _stale(obj, [os.path.join(CSRC, src)] + hdrs):
            todo.append((src, extra + flag))
    logs = []
    if todo:
        with cf.ThreadPoolExecutor(max_workers=jobs or min(len(todo), os.cpu_count() or 4)) as ex:
            for obj, log in ex.map(lambda a: _compile(a[0], a[1], verbose, bdir), todo):
                logs.append((obj, log))
    objs = [os.path.join(bdir, s.replace(".cu", ".o")) for s, _ in SOURCES]
    LIB_ = lib
    if force or todo or _stale(LIB_, objs):
        tmp = LIB_ + ".tmp%d" % os.getpid()
        cmd = [nvcc(), "-shared", "-cudart", "shared", "-o", tmp] + objs + ARCH
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n%s\n%s" % (" ".join(cmd), r.stderr))
        os.replace(tmp, LIB_)
    if verbose:
        for obj, log in logs:
            sys.stderr.write("== %s\n%s" % (os.path.basename(obj), log))
    return LIB_


if __name__ == "__main__":
    path = build(force="--force" in sys.argv, verbose="-v" in sys.argv,
                 check="--check" in sys.argv)
    print(path)
