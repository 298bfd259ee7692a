"""In-tree build of liboceano_gpu.so for sm_103a (nvcc, no cmake).

The four degree instantiations of the fused stage kernel, the auxiliary
kernels and the C ABI compile as separate translation units in parallel and
link into one shared library next to this file.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "liboceano_gpu.so")
LIB_CHECKED = os.path.join(HERE, "liboceano_gpu_checked.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
         "--expt-relaxed-constexpr", "-I" + INCLUDE]


def _nvcc() -> str:
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _sources():
    units = []
    for rule in (0, 1):  # cell Gauss rule: floor(1.5 p) + 1 or p + 1 points per direction
        for p in (1, 2, 3, 4):
            # FP32 bulk of the mixed form: flush-to-zero and approximate division and
            # square root (affects single precision only; the FP64 form is IEEE)
            units.append((os.path.join(CSRC, "oc_stage_inst.cu"),
                          f"oc_stage_p{p}" + ("_r1" if rule else "") + ".o",
                          [f"-DOC_DEGREE={p}", f"-DOC_CELL_RULE={rule}", "-ftz=true",
                           "-prec-div=false", "-prec-sqrt=false"]))
    for v in (0, 1, 2):
        units.append((os.path.join(CSRC, "oc_stage_hp.cu"), f"oc_stage_hp_v{v}.o",
                      [f"-DOC_HP_VARIANT={v}", "-ftz=true", "-prec-div=false",
                       "-prec-sqrt=false"]))
    units.append((os.path.join(CSRC, "oc_face.cu"), "oc_face.o", []))
    units.append((os.path.join(CSRC, "oc_aux.cu"), "oc_aux.o", []))
    units.append((os.path.join(CSRC, "oc_api.cu"), "oc_api.o", []))
    units.append((os.path.join(CSRC, "oc_noalloc.cu"), "oc_noalloc.o", []))
    units.append((os.path.join(CSRC, "oc_mlp.cu"), "oc_mlp.o", []))
    return units


def _newest_source() -> float:
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    files.append(os.path.join(INCLUDE, "oceano_gpu.h"))
    files.append(os.path.abspath(__file__))
    return max(os.path.getmtime(f) for f in files)


def build(force: bool = False, verbose: bool = False, extra=(), bounds_check: bool = False) -> str:
    """Compile the library; bounds_check=True builds the bounds-checked variant
    (OC_BOUNDS_CHECK: every index read from a mesh table range-checked into the
    device error word) as liboceano_gpu_checked.so, in its own build folder."""
    lib, build_dir = (LIB_CHECKED, BUILD + "_checked") if bounds_check else (LIB, BUILD)
    if bounds_check:
        extra = [*extra, "-DOC_BOUNDS_CHECK"]
    if not force and os.path.exists(lib) and os.path.getmtime(lib) >= _newest_source():
        return lib
    os.makedirs(build_dir, exist_ok=True)
    nvcc = _nvcc()
    jobs = []
    for src, obj, defs in _sources():
        cmd = [nvcc, *ARCH, *FLAGS, *defs, *extra, "-c", src, "-o", os.path.join(build_dir, obj)]
        jobs.append(cmd)

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        return cmd, r

    with cf.ThreadPoolExecutor(max_workers=min(16, os.cpu_count() or 2)) as ex:
        for cmd, r in ex.map(run, jobs):
            if verbose or r.returncode:
                print(" ".join(cmd))
                print(r.stdout[-4000:], r.stderr[-8000:])
            if r.returncode:
                raise RuntimeError(f"nvcc failed: {cmd[-3]}")
    objs = [os.path.join(build_dir, o) for _, o, _ in _sources()]
    tmp = lib + ".tmp"
    subprocess.check_call([nvcc, *ARCH, "-shared", "-o", tmp, *objs, "-lcudart"])
    os.replace(tmp, lib)
    return lib


if __name__ == "__main__":
    import sys
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv,
                extra=["-Xptxas", "-v"] if "--ptxas" in sys.argv else [],
                bounds_check="--bounds-check" in sys.argv))
