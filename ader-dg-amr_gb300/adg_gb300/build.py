"""Build the sm_103a shared library of the ADER-DG element path, in-tree.

Steps: generate the per-(D, P) element operator headers, compile one object
per configuration plus the host context in parallel with nvcc, link
adg_gb300/_lib/libadg.so.  No cmake; only nvcc and the Python interpreter.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
PROJ_DIR = os.path.dirname(PKG_DIR)  # ader-dg-amr_gb300/
REPO_DIR = os.path.dirname(PROJ_DIR)
CSRC = os.path.join(PROJ_DIR, "csrc")
INCLUDE = os.path.join(REPO_DIR, "include")
BUILD = os.path.join(PROJ_DIR, "_build")
GEN = os.path.join(BUILD, "gen")
LIB_DIR = os.path.join(PKG_DIR, "_lib")
LIB_PATH = os.path.join(LIB_DIR, "libadg.so")

CONFIGS = [(2, 1), (2, 2), (2, 3), (3, 1), (3, 2), (2, 4), (2, 5), (2, 6), (3, 3)]
# (D, P) built with the plain FP64 path only (no learned-seed predictor modes,
# one elements-per-block choice): the seed network's layers do not fit its
# fused kernel there, and it keeps their large generated units quick to build
LITE = {(2, 4), (2, 5), (2, 6), (3, 3)}
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
                     "--expt-relaxed-constexpr", "-I", INCLUDE, "-I", CSRC, "-I", GEN]


def _nvcc():
    p = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(p):
        raise RuntimeError("nvcc not found")
    return p


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("command failed: " + " ".join(cmd) + "\n" + r.stdout)
    return r.stdout


def _sources_newer(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def build(verbose=False, extra_flags=()):
    os.makedirs(GEN, exist_ok=True)
    os.makedirs(LIB_DIR, exist_ok=True)
    gen_script = os.path.join(CSRC, "gen_element.py")
    stale = [(d, p) for d, p in CONFIGS if _sources_newer(os.path.join(GEN, f"elem_D{d}P{p}.cuh"), [gen_script])]
    if stale:  # one generator process per configuration, in parallel
        with cf.ThreadPoolExecutor(max_workers=max(1, min(len(stale), os.cpu_count() or 4))) as ex:
            list(ex.map(_run, [[sys.executable, gen_script, "--out-dir", GEN, "--configs", f"{d}:{p}"]
                               for d, p in stale]))
    nvcc = _nvcc()
    common_deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".hpp", ".cu", ".h"))]
    common_deps.append(os.path.join(INCLUDE, "adg.h"))
    jobs = []
    objs = []
    for d, p in CONFIGS:
        obj = os.path.join(BUILD, f"adg_inst_D{d}P{p}.o")
        objs.append(obj)
        deps = common_deps + [os.path.join(GEN, f"elem_D{d}P{p}.cuh")]
        if _sources_newer(obj, deps):
            jobs.append([nvcc, *NVCC_FLAGS, *extra_flags, "-c", os.path.join(CSRC, "adg_inst.cu"), "-o", obj,
                         f"-DADG_D={d}", f"-DADG_HDR=\"elem_D{d}P{p}.cuh\"", f"-DADG_NS=gen_D{d}P{p}",
                         f"-DADG_FACTORY=kernels_D{d}P{p}", f"-DADG_LITE={int((d, p) in LITE)}"])
    for src in ("adg_ctx.cu", "adg_amr.cu", "adg_noalloc.cu"):
        path = os.path.join(CSRC, src)
        if not os.path.exists(path):
            continue
        obj = os.path.join(BUILD, src.replace(".cu", ".o"))
        objs.append(obj)
        if _sources_newer(obj, common_deps):
            jobs.append([nvcc, *NVCC_FLAGS, *extra_flags, "-c", path, "-o", obj])
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        outs = list(ex.map(_run, jobs))
    if verbose:
        for o in outs:
            if o.strip():
                print(o)
    if jobs or not os.path.exists(LIB_PATH):
        _run([nvcc, *ARCH, "-shared", "-o", LIB_PATH, *objs])
    return LIB_PATH


if __name__ == "__main__":
    print(build(verbose=True))
