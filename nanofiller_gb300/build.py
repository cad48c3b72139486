"""Builds libnanofiller_gb300.so (sm_103a) in-tree, in nanofiller_gb300/_build/.

Each .cu translation unit is compiled in parallel with nvcc, then linked into one
shared library with a static CUDA runtime; the command-line front end
(_build/nanofiller, cli/nanofiller.cpp) is linked against it. Host code is compiled with
-ffp-contract=off so the host half of the seeded stream matches the device bits
on x86-64 and aarch64 alike.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libnanofiller_gb300.so")
CLI = os.path.join(OUT, "nanofiller")
SOURCES = ["nf_generate.cu", "nf_contacts.cu", "nf_solve.cu", "nf_internal.cu", "nf_ac.cu", "nf_prune.cu", "nf_stats.cu", "nf_align.cu", "nf_api.cu", "nf_alloc.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _flags(verbose_ptxas=False):
    f = ARCH + ["-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr",
                "-Xcompiler", "-fPIC,-ffp-contract=off,-fno-fast-math",
                "-I", os.path.join(HERE, "..", "include")]
    if verbose_ptxas:
        f += ["-Xptxas", "-v"]
    return f


def _stale():
    if not os.path.exists(LIB) or not os.path.exists(CLI):
        return True
    t = min(os.path.getmtime(LIB), os.path.getmtime(CLI))
    deps = [os.path.join(SRC, f) for f in os.listdir(SRC)]
    deps.append(os.path.join(HERE, "cli", "nanofiller.cpp"))
    deps.append(os.path.join(HERE, "..", "include", "nanofiller_gb300.h"))
    deps.append(os.path.abspath(__file__))
    return any(os.path.getmtime(d) > t for d in deps)


def build(force=False, verbose_ptxas=False, jobs=None):
    """Compile the library if any source is newer than it. Returns its path."""
    if not force and not _stale():
        return LIB
    os.makedirs(OUT, exist_ok=True)
    nv = nvcc()
    objs = []

    def one(src):
        obj = os.path.join(OUT, src.replace(".cu", ".o"))
        cmd = [nv, "-c", os.path.join(SRC, src), "-o", obj] + _flags(verbose_ptxas)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src}:\n{r.stderr}")
        return obj, r.stderr

    with cf.ThreadPoolExecutor(max_workers=jobs or len(SOURCES)) as ex:
        for obj, log in ex.map(one, SOURCES):
            objs.append(obj)
            if verbose_ptxas and log:
                sys.stderr.write(log)
    tmp = LIB + ".tmp"
    cmd = [nv, "-shared", "-o", tmp] + objs + ARCH + ["-Xcompiler", "-fPIC", "-cudart", "static"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr}")
    os.replace(tmp, LIB)
    # Command-line front end, linked against the library next to it.
    cxx = shutil.which("g++") or "g++"
    cmd = [cxx, "-O2", "-std=c++17", "-I", os.path.join(HERE, "..", "include"),
           os.path.join(HERE, "cli", "nanofiller.cpp"), "-o", CLI + ".tmp", "-L", OUT,
           "-l:libnanofiller_gb300.so", "-Wl,-rpath,$ORIGIN"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"command-line front end failed to build:\n{r.stderr}")
    os.replace(CLI + ".tmp", CLI)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose_ptxas="-v" in sys.argv))
