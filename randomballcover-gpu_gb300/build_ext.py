"""Build librbcgb.so in-tree: every csrc/*.cu / *.cpp compiled for sm_103a with
nvcc (in parallel), linked into one shared library next to this file.  The
legacy C++ API is compiled a second time with RBC_REAL_DOUBLE (the reference's
real = double build) and linked with the same objects into librbcgb_f64.so.

    python randomballcover-gpu_gb300/build_ext.py [--force]
"""
import concurrent.futures as cf
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "librbcgb.so")
LIB64 = os.path.join(HERE, "librbcgb_f64.so")
LEGACY = os.path.join(CSRC, "legacy.cu")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

NVCC = os.environ.get("NVCC", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# -ffp-contract=off: host code that restates the reference's distance
# (bruteCPU, distVec) must round each multiply and add on its own on every host.
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-ffp-contract=off", f"-I{INCLUDE}"]


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cu", ".cpp")))


def headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    hs += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE) if f.endswith(".h")]
    return hs


def _compile(job):
    src, defs = job if isinstance(job, tuple) else (job, [])
    obj = os.path.join(BUILD, os.path.basename(src) + ("".join(d.replace("-D", ".") for d in defs)) + ".o")
    newest_dep = max([os.path.getmtime(src)] + [os.path.getmtime(h) for h in headers()])
    if os.path.exists(obj) and os.path.getmtime(obj) >= newest_dep:
        return obj, None
    cmd = [NVCC] + ARCH + COMMON + defs + ["-c", src, "-o", obj]
    if src.endswith(".cpp"):
        cmd = [NVCC] + COMMON + ["-x", "c++", "-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        return obj, f"{' '.join(cmd)}\n{r.stdout}{r.stderr}"
    return obj, None


def build(force=False, verbose=False):
    os.makedirs(BUILD, exist_ok=True)
    if force:
        for f in os.listdir(BUILD):
            os.remove(os.path.join(BUILD, f))
    srcs = sources()
    jobs = srcs + [(LEGACY, ["-DRBC_REAL_DOUBLE"])]
    with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
        results = list(ex.map(_compile, jobs))
    errors = [e for _, e in results if e]
    if errors:
        raise RuntimeError("nvcc failed:\n" + "\n".join(errors))
    objs = [o for o, _ in results[:len(srcs)]]
    legacy_obj = objs[srcs.index(LEGACY)]
    objs64 = [o for o in objs if o != legacy_obj] + [results[-1][0]]
    for lib, parts in ((LIB, objs), (LIB64, objs64)):
        if not (os.path.exists(lib) and os.path.getmtime(lib) >= max(os.path.getmtime(o) for o in parts)):
            cmd = [NVCC] + ARCH + ["-shared", "-o", lib] + parts
            r = subprocess.run(cmd, capture_output=True, text=True)
            if r.returncode != 0:
                raise RuntimeError(f"link failed:\n{' '.join(cmd)}\n{r.stdout}{r.stderr}")
    build_cli()
    if verbose:
        print("built", LIB, "and", CLI)
    return LIB


CLI = os.path.join(HERE, "testRBC")
CLI_SRC = os.path.join(HERE, "cli", "testRBC.cu")


def build_cli():
    """The testRBC command-line driver, linked against the library (rpath $ORIGIN)."""
    if os.path.exists(CLI) and os.path.getmtime(CLI) >= max(os.path.getmtime(CLI_SRC), os.path.getmtime(LIB)):
        return CLI
    cmd = [NVCC, "-O2", "-std=c++17", f"-I{INCLUDE}", CLI_SRC, "-o", CLI, f"-L{HERE}", "-lrbcgb",
           "-Xlinker=-rpath=$ORIGIN"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"CLI build failed:\n{' '.join(cmd)}\n{r.stdout}{r.stderr}")
    return CLI


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
