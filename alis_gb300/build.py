"""Build the GB300 ALiS engine in-tree.

Products (all under alis_gb300/lib/, git-ignored):
  libalis_gb300.so   the ALiS C API backed by the CUDA engine (sm_103a)
  libalis_gb300.a    the same as a static archive (link with -lcudart)
and, when asked, the oracle build used by the tests:
  oracle/build/liboracle_alis.a   host setup layer + CPU restatement

Host C is compiled with -ffp-contract=off so the setup arithmetic rounds
exactly like the reference on any host ISA (the GPU machine is aarch64,
whose compilers otherwise fuse multiply-adds).  The Yee and phaser
kernels are compiled with -fmad=false for the same reason.
"""
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "alis_gb300")
HOST = os.path.join(PKG, "csrc", "host")
GPU = os.path.join(PKG, "csrc", "gpu")
INC = os.path.join(ROOT, "include")
LIB = os.path.join(PKG, "lib")
ORACLE = os.path.join(ROOT, "oracle")
ORACLE_BUILD = os.path.join(ORACLE, "build")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CFLAGS = ["-std=gnu99", "-O3", "-fPIC", "-fopenmp", "-ffp-contract=off", "-w",
          "-I" + INC, "-I" + HOST]
HOST_SOURCES = ["world.c", "object.c", "shapes.c", "source.c", "phaser.c", "farfld.c",
                "fields.c", "output.c", "slices.c", "timer.c"]
# (source, exact-rounding)
CUDA_SOURCES = [("world.cu", True), ("phaser.cu", True), ("voxel.cu", True), ("farfield.cu", False)]


def _cuda_home():
    for c in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if c and os.path.exists(os.path.join(c, "bin", "nvcc")):
            return c
    nvcc = shutil.which("nvcc")
    return os.path.dirname(os.path.dirname(nvcc)) if nvcc else "/usr/local/cuda"


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode:
        raise RuntimeError("build failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
    return r


def _newer(target, sources):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(s) > t for s in sources)


def _objdir(name):
    d = os.path.join(LIB, "obj", name)
    os.makedirs(d, exist_ok=True)
    return d


def build_engine(force=False, verbose=False, nvcc_extra=()):
    """Compile the CUDA engine into alis_gb300/lib/libalis_gb300.{so,a}.
    nvcc_extra: further nvcc arguments (e.g. -D tuning macros)."""
    cuda = _cuda_home()
    nvcc = os.path.join(cuda, "bin", "nvcc")
    os.makedirs(LIB, exist_ok=True)
    od = _objdir("engine")
    headers = [os.path.join(INC, h) for h in os.listdir(INC)] + \
        [os.path.join(HOST, "engine.h"), os.path.join(GPU, "common.cuh")]
    jobs = []
    for s in HOST_SOURCES:
        src, obj = os.path.join(HOST, s), os.path.join(od, s + ".o")
        if force or _newer(obj, [src] + headers):
            jobs.append(["gcc"] + CFLAGS + ["-c", src, "-o", obj])
    src, obj = os.path.join(GPU, "gpu_backend.c"), os.path.join(od, "gpu_backend.c.o")
    if force or _newer(obj, [src] + headers):
        jobs.append(["gcc"] + CFLAGS + ["-c", src, "-o", obj])
    for s, exact in CUDA_SOURCES:
        src, obj = os.path.join(GPU, s), os.path.join(od, s + ".o")
        if force or _newer(obj, [src] + headers):
            cmd = [nvcc] + ARCH + ["-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC",
                                   "-I" + INC, "-I" + GPU, "-c", src, "-o", obj]
            cmd += ["-fmad=false"] if exact else ["-fmad=true"]
            if os.environ.get("ALISGPU_PTXAS_VERBOSE"):
                cmd += ["-Xptxas", "-v"]
            jobs.append(cmd + list(nvcc_extra))
    with ThreadPoolExecutor(max_workers=os.cpu_count() or 4) as ex:
        for r in ex.map(_run, jobs):
            if verbose and (r.stdout or r.stderr):
                sys.stderr.write(r.stdout + r.stderr)
    objs = [os.path.join(od, s + ".o") for s in HOST_SOURCES] + [os.path.join(od, "gpu_backend.c.o")] + \
        [os.path.join(od, s + ".o") for s, _ in CUDA_SOURCES]
    so = os.path.join(LIB, "libalis_gb300.so")
    if force or _newer(so, objs):
        _run(["g++", "-shared", "-o", so] + objs +
             ["-L" + os.path.join(cuda, "lib64"), "-Wl,-rpath," + os.path.join(cuda, "lib64"),
              "-lcudart", "-lgomp", "-lm"])
    ar = os.path.join(LIB, "libalis_gb300.a")
    if force or _newer(ar, objs):
        if os.path.exists(ar):
            os.remove(ar)
        _run(["ar", "rcs", ar] + objs)
    return so


FP64_HEADER = os.path.join(ORACLE, "fp64.h")


def build_oracle(force=False, fp64=False):
    """Compile the CPU oracle (host setup layer + restated stepper).
    fp64: the same sources with float read as double (oracle/fp64.h), the
    FP64 run against which the error of the FP32 arithmetic is stated."""
    os.makedirs(ORACLE_BUILD, exist_ok=True)
    od = os.path.join(ORACLE_BUILD, "obj64" if fp64 else "obj")
    os.makedirs(od, exist_ok=True)
    headers = [os.path.join(INC, h) for h in os.listdir(INC)] + [os.path.join(HOST, "engine.h")]
    flags = CFLAGS + (["-include", FP64_HEADER] if fp64 else [])
    if fp64:
        headers.append(FP64_HEADER)
    srcs = [os.path.join(HOST, s) for s in HOST_SOURCES] + [os.path.join(ORACLE, "cpu_step.c")]
    jobs, objs = [], []
    for src in srcs:
        obj = os.path.join(od, os.path.basename(src) + ".o")
        objs.append(obj)
        if force or _newer(obj, [src] + headers):
            jobs.append(["gcc"] + flags + ["-c", src, "-o", obj])
    with ThreadPoolExecutor(max_workers=os.cpu_count() or 4) as ex:
        list(ex.map(_run, jobs))
    ar = os.path.join(ORACLE_BUILD, "liboracle_alis64.a" if fp64 else "liboracle_alis.a")
    if force or _newer(ar, objs):
        if os.path.exists(ar):
            os.remove(ar)
        _run(["ar", "rcs", ar] + objs)
    return ar


def reference_root():
    """The reference checkout as oracle/build_ref.sh locates it (its
    argument-free form: $ALIS_REFERENCE or the build container's
    checkout), or None where there is none (the GPU machine)."""
    r = subprocess.run(["sh", os.path.join(ORACLE, "build_ref.sh"), "--locate"], capture_output=True, text=True)
    path = r.stdout.strip()
    return path if r.returncode == 0 and os.path.isdir(os.path.join(path, "src")) else None


def build_reference(force=False):
    """Build the reference library from its own sources (only where the
    reference checkout exists; used to pin the oracle)."""
    ref = reference_root()
    if ref is None:
        return None
    lib = os.path.join(ORACLE, "_ref", "libalis_ref.a")
    if force or not os.path.exists(lib):
        _run(["sh", os.path.join(ORACLE, "build_ref.sh"), ref])
    return lib


def link_program(source, out, against="engine", extra=()):
    """Compile a C program written against the ALiS API and link it with
    the engine ("engine"), the oracle ("oracle"), the oracle's FP64 build
    ("oracle64") or the reference ("reference")."""
    cuda = _cuda_home()
    os.makedirs(os.path.dirname(out), exist_ok=True)
    base = ["gcc", "-std=gnu99", "-O2", "-fopenmp", "-ffp-contract=off", "-w", source, "-o", out]
    if against == "engine":
        cmd = base[:1] + ["-I" + INC] + base[1:] + ["-L" + LIB, "-lalis_gb300", "-Wl,-rpath," + LIB,
                                                    "-L" + os.path.join(cuda, "lib64"), "-lcudart", "-lm"]
    elif against == "oracle":
        cmd = base[:1] + ["-I" + INC] + base[1:] + [os.path.join(ORACLE_BUILD, "liboracle_alis.a"), "-lm"]
    elif against == "oracle64":
        cmd = base[:1] + ["-include", FP64_HEADER, "-I" + INC] + base[1:] + \
            [os.path.join(ORACLE_BUILD, "liboracle_alis64.a"), "-lm"]
    elif against == "reference":
        ref = reference_root()
        if ref is None:
            raise RuntimeError("no reference checkout (oracle/build_ref.sh --locate)")
        cmd = ["gcc", "-std=c99", "-O2", "-fopenmp", "-ffp-contract=off", "-w", "-I" + os.path.join(ref, "src"),
               source, "-o", out, os.path.join(ORACLE, "_ref", "libalis_ref.a"), "-lm"]
    else:
        raise ValueError(against)
    _run(cmd + list(extra))
    return out


if __name__ == "__main__":
    print(build_engine(force="--force" in sys.argv, verbose=True))
    print(build_oracle(force="--force" in sys.argv))
