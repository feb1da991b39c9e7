"""Builds libdmgb.so in-tree with nvcc for sm_103a (GB300).

The library is a plain C ABI (include/dmgb.h); Python loads it with ctypes.
Objects and the shared library go to seismicmesh_gb300/lib/ (git-ignored).
"""
import concurrent.futures
import os
import shutil
import subprocess

PKG = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(PKG, "csrc")
LIBDIR = os.path.join(PKG, "lib")
LIBNAME = "libdmgb.so"

SOURCES = [
    "dm_common.cu",
    "dm_delaunay.cu",
    "dm_mesh.cu",
    "dm_sizing.cu",
    "dm_topo.cu",
    "dm_iso.cu",
    "dm_mlp.cu",
    "dm_capi.cu",
]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = [
    "-O3",
    "-lineinfo",
    "-std=c++17",
    "-Xcompiler",
    "-fPIC,-O2,-ffp-contract=off",
    "--expt-relaxed-constexpr",
]


def nvcc_path():
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libdmgb.so")


def library_path():
    return os.path.join(LIBDIR, LIBNAME)


def _needs_rebuild(obj, deps):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(d) > t for d in deps)


def build_library(verbose=False, force=False, extra_flags=()):
    nvcc = nvcc_path()
    extra_flags = (*extra_flags, *os.environ.get("DMGB_NVCC_FLAGS", "").split())
    objdir = os.path.join(LIBDIR, "obj")
    os.makedirs(objdir, exist_ok=True)
    # objects built with other flags are rebuilt
    stamp = os.path.join(objdir, "flags.txt")
    flags_id = " ".join([*ARCH, *NVCC_FLAGS, *extra_flags])
    if not os.path.exists(stamp) or open(stamp).read() != flags_id:
        force = True
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cuh")]
    headers.append(os.path.join(PKG, "..", "include", "dmgb.h"))
    jobs = []
    for src in SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(objdir, src.replace(".cu", ".o"))
        if force or _needs_rebuild(o, [s] + headers):
            cmd = [nvcc, *ARCH, *NVCC_FLAGS, *extra_flags, "-c", s, "-o", o]
            jobs.append((src, cmd))

    def run(job):
        src, cmd = job
        r = subprocess.run(cmd, capture_output=True, text=True)
        return src, cmd, r

    with concurrent.futures.ThreadPoolExecutor(max_workers=max(1, len(jobs))) as ex:
        for src, cmd, r in ex.map(run, jobs):
            if verbose or r.returncode != 0:
                print(" ".join(cmd))
                print(r.stdout, r.stderr)
            if r.returncode != 0:
                raise RuntimeError(f"nvcc failed on {src}:\n{r.stderr}")
    lib = library_path()
    objs = [os.path.join(objdir, s.replace(".cu", ".o")) for s in SOURCES]
    if force or jobs or not os.path.exists(lib):
        cmd = [nvcc, *ARCH, "-shared", "-o", lib + ".tmp", *objs]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stderr}")
        os.replace(lib + ".tmp", lib)
    with open(stamp, "w") as fh:
        fh.write(flags_id)
    return lib


if __name__ == "__main__":
    print(build_library(verbose=True))
