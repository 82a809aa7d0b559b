"""In-tree build of the native parts: the sm_103a CUDA library (liblgpu.so)
and the synthetic workload generator (liblgsynth.so).  No cmake: nvcc and
gcc are called directly, translation units compiled in parallel."""
import os
import subprocess
import concurrent.futures as cf

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)                      # umd-letkf_gb300/
REPO = os.path.dirname(ROOT)
CSRC = os.path.join(ROOT, "csrc")
SYNTH = os.path.join(ROOT, "synth")
INCLUDE = os.path.join(REPO, "include")
BUILD = os.path.join(ROOT, "_build")
LGPU = os.path.join(ROOT, "liblgpu.so")
LGSYNTH = os.path.join(SYNTH, "liblgsynth.so")

ARCH = "-gencode=arch=compute_103a,code=sm_103a"
CU_SOURCES = ["lgpu_api.cu", "lgpu_index.cu", "lgpu_gram.cu", "lgpu_gram_tc.cu", "lgpu_eig.cu", "lgpu_update.cu",
              "lgpu_update_tc.cu", "lgpu_noalloc.cu", "lgpu_prep.cu", "lgpu_mlp.cu", "lgpu_learn.cu", "lgpu_ncio.cpp"]
NVCC_FLAGS = ["-O3", "-std=c++17", ARCH, "-lineinfo", "-Xcompiler", "-fPIC",
              "-prec-div=true", "-prec-sqrt=true", "-ftz=false",
              "-Xptxas", "-O3", "-I", INCLUDE, "-I", CSRC]


def _nvcc():
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if c and (os.path.isabs(c) and os.path.exists(c) or not os.path.isabs(c)):
            return c
    return "nvcc"


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def _headers():
    hs = [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE) if f.endswith(".h")]
    hs += [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    return hs


def build_synth(force=False):
    src = os.path.join(SYNTH, "lgsynth.c")
    if force or _stale(LGSYNTH, [src, os.path.join(SYNTH, "lgsynth.h")]):
        subprocess.check_call(["gcc", "-O2", "-std=c11", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
                               "-o", LGSYNTH, src, "-lm"])
    return LGSYNTH


def build_lgpu(force=False, verbose=False):
    os.makedirs(BUILD, exist_ok=True)
    nvcc = _nvcc()
    hdrs = _headers()
    objs, jobs = [], []
    for s in CU_SOURCES:
        src = os.path.join(CSRC, s)
        obj = os.path.join(BUILD, os.path.splitext(s)[0] + ".o")
        objs.append(obj)
        if force or _stale(obj, [src] + hdrs):
            cmd = [nvcc] + NVCC_FLAGS + ["-c", src, "-o", obj]
            if verbose:
                cmd += ["-Xptxas", "-v"]
            jobs.append(cmd)
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(8, len(jobs))) as ex:
            futs = [ex.submit(subprocess.run, j, capture_output=True, text=True) for j in jobs]
            for f, j in zip(futs, jobs):
                r = f.result()
                if verbose and r.stderr:
                    print(r.stderr)
                if r.returncode != 0:
                    raise RuntimeError("nvcc failed: %s\n%s%s" % (" ".join(j), r.stdout, r.stderr))
    if force or jobs or not os.path.exists(LGPU):
        subprocess.check_call([nvcc, ARCH, "-shared", "-o", LGPU] + objs + ["-lcudart"])
    return LGPU


def synth_lib_path():
    if not os.path.exists(LGSYNTH):
        build_synth()
    return LGSYNTH


def lgpu_lib_path():
    return LGPU


def build_all(force=False, verbose=False):
    build_synth(force)
    build_lgpu(force, verbose)
