"""In-tree build of the solver libraries, the dgalerkin executable and the
CPU oracle.

Outputs (git-ignored, rebuilt on every machine):
  dgfem-acoustic_gb300/_build/libdgfem_host.so   host front end (no CUDA)
  dgfem-acoustic_gb300/_build/libdgfem_gb300.so  GPU solver (C ABI)
  dgfem-acoustic_gb300/_build/dgalerkin          drop-in driver executable
  oracle/_build/librefcpu.so                     CPU oracle (test infrastructure)

CUDA code is compiled for sm_103a only. Translation units are compiled in
parallel and skipped when their object is newer than every source/header.
"""
import concurrent.futures as cf
import glob
import os
import shutil
import subprocess

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
OUT = os.path.join(PKG, "_build")
OBJ = os.path.join(OUT, "obj")
ORACLE = os.path.join(ROOT, "oracle")
INCLUDE = os.path.join(ROOT, "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CXXFLAGS = ["-O3", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall", "-Wno-unused-function"]
NVCCFLAGS = ARCH + ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
                    "-I" + INCLUDE]

HOST_SRC = ["mshio.cpp", "host_mesh.cpp", "host_api.cpp", "refelem.cpp", "config.cpp", "formula.cpp", "outputs.cpp", "quadrature.cpp"]
GPU_SRC = ["capi.cu", "setup.cu", "stage_f32_2d.cu", "stage_f32_3d.cu", "stage_f64_2d.cu", "stage_f64_3d.cu", "stage_1d.cu", "stage_tc.cu", "stage_tc2.cu", "stage_tc3.cu", "stage3.cu", "stage4.cu", "stage_multi.cu", "curved.cu", "vtu_writer.cu", "noalloc.cu", "batch.cu", "mlp.cu"]
GPU_HOST_SRC = ["refelem.cpp", "quadrature.cpp"]


def _nvcc():
    for c in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _headers():
    hs = glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(CSRC, "*.cuh"))
    hs += glob.glob(os.path.join(INCLUDE, "*.h"))
    return hs


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: %s\n%s" % (" ".join(cmd), r.stdout))
    return r.stdout


def _compile(src, obj, cuda):
    deps = [src] + _headers()
    if not _stale(obj, deps):
        return obj
    os.makedirs(os.path.dirname(obj), exist_ok=True)
    if cuda:
        _run([_nvcc()] + NVCCFLAGS + ["-c", src, "-o", obj])
    else:
        _run(["g++"] + CXXFLAGS + ["-I" + INCLUDE, "-c", src, "-o", obj])
    return obj


def build(verbose=False):
    os.makedirs(OBJ, exist_ok=True)
    jobs = []
    with cf.ThreadPoolExecutor(max_workers=max(2, min(12, os.cpu_count() or 4))) as ex:
        for s in [h for h in HOST_SRC if os.path.exists(os.path.join(CSRC, h))]:
            jobs.append(ex.submit(_compile, os.path.join(CSRC, s), os.path.join(OBJ, "host_" + s + ".o"), False))
        for s in GPU_SRC:
            jobs.append(ex.submit(_compile, os.path.join(CSRC, s), os.path.join(OBJ, "gpu_" + s + ".o"), True))
        oracle_so = os.path.join(ORACLE, "_build", "librefcpu.so")
        osrc = os.path.join(ORACLE, "refcpu.cpp")
        if _stale(oracle_so, [osrc, os.path.join(ORACLE, "refcpu.h")]):
            os.makedirs(os.path.dirname(oracle_so), exist_ok=True)
            jobs.append(ex.submit(_run, ["g++", "-O3", "-std=c++17", "-fPIC", "-shared", "-fopenmp",
                                         "-ffp-contract=off", "-Wall", osrc, "-o", oracle_so]))
        for j in jobs:
            j.result()
    host_objs = [os.path.join(OBJ, "host_" + s + ".o") for s in HOST_SRC if os.path.exists(os.path.join(CSRC, s))]
    host_so = os.path.join(OUT, "libdgfem_host.so")
    if _stale(host_so, host_objs):
        _run(["g++", "-shared", "-o", host_so] + host_objs)
    gpu_objs = [os.path.join(OBJ, "gpu_" + s + ".o") for s in GPU_SRC]
    gpu_objs += [os.path.join(OBJ, "host_" + s + ".o") for s in GPU_HOST_SRC]
    gpu_so = os.path.join(OUT, "libdgfem_gb300.so")
    if _stale(gpu_so, gpu_objs):
        _run([_nvcc()] + ARCH + ["-shared", "-o", gpu_so] + gpu_objs)
    exe = os.path.join(OUT, "dgalerkin")
    main_src = os.path.join(CSRC, "dgalerkin.cpp")
    if os.path.exists(main_src) and _stale(exe, [main_src, host_so, gpu_so] + _headers()):
        _run(["g++"] + CXXFLAGS + ["-I" + INCLUDE, main_src, "-o", exe, "-L" + OUT,
                                   "-ldgfem_host", "-ldgfem_gb300", "-Wl,-rpath,$ORIGIN"])
    return dict(host=host_so, gpu=gpu_so, exe=exe, oracle=oracle_so)


if __name__ == "__main__":
    print(build())
