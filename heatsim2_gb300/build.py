"""Build libhs2g.so in-tree with nvcc for sm_103a (GB300).

    python -m heatsim2_gb300.build

Translation units are compiled in parallel and linked against the shared CUDA runtime.
"""
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
ROOT = os.path.dirname(HERE)
OUT = os.path.join(HERE, "libhs2g.so")
BUILD_DIR = os.path.join(HERE, "_build")
SOURCES = ["hs2g_api.cu", "hs2g_compile.cu", "hs2g_sweep.cu", "hs2g_lines.cu", "hs2g_static.cu", "hs2g_batch.cu",
           "hs2g_adjoint.cu", "hs2g_sources.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc_path():
    cand = shutil.which("nvcc")
    if cand:
        return cand
    cand = "/usr/local/cuda/bin/nvcc"
    if os.path.exists(cand):
        return cand
    raise RuntimeError("nvcc not found")


def _cuda_lib_dir(nvcc):
    root = os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))
    for sub in ("lib64", "lib", "targets/sbsa-linux/lib", "targets/x86_64-linux/lib"):
        p = os.path.join(root, sub)
        if os.path.exists(os.path.join(p, "libcudart.so")):
            return p
    return os.path.join(root, "lib64")


def build(force=False, verbose=False):
    nvcc = nvcc_path()
    os.makedirs(BUILD_DIR, exist_ok=True)
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [os.path.join(ROOT, "include", "hs2g.h")]
    newest = max(os.path.getmtime(p) for p in deps if os.path.exists(p))
    if not force and os.path.exists(OUT) and os.path.getmtime(OUT) >= newest:
        return OUT
    common = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
                     "-I" + os.path.join(ROOT, "include")]
    procs = []
    objs = []
    for src in SOURCES:
        obj = os.path.join(BUILD_DIR, src.replace(".cu", ".o"))
        objs.append(obj)
        cmd = [nvcc, "-c", os.path.join(CSRC, src), "-o", obj] + common
        if verbose:
            print(" ".join(cmd))
        procs.append((src, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
    errors = []
    for src, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            errors.append("%s:\n%s" % (src, out.decode(errors="replace")))
    if errors:
        raise RuntimeError("nvcc failed:\n" + "\n".join(errors))
    libdir = _cuda_lib_dir(nvcc)
    tmp = OUT + ".tmp"
    subprocess.check_call([nvcc, "-shared"] + ARCH + ["-o", tmp] + objs +
                          ["-cudart", "shared", "-Xlinker", "-rpath," + libdir])
    os.replace(tmp, OUT)
    return OUT


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
