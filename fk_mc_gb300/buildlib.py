"""Build the sm_103a CUDA library libfkg.so (the C ABI of include/fkg.h).

The library is compiled in-tree into fk_mc_gb300/_build/ with nvcc for
sm_103a only; the translation units are compiled in parallel and linked with
the static CUDA runtime, so the .so has no dependency on torch.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libfkg.so")
HOST_LIB = os.path.join(OUT, "libfk_mc_host.so")
HOST_SRCS = [os.path.join(HERE, "host", f) for f in ("fkh_capi.cpp", "fkh_stats.cpp")]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
           "-I", os.path.join(ROOT, "include")]


def nvcc():
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def _headers():
    return [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))] + \
        [os.path.join(ROOT, "include", f) for f in os.listdir(os.path.join(ROOT, "include"))]


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force=False, verbose=False, extra=()):
    os.makedirs(OUT, exist_ok=True)
    nv = nvcc()
    hdrs = _headers()
    objs = []
    jobs = []
    for src in sources():
        obj = os.path.join(OUT, os.path.basename(src)[:-3] + ".o")
        objs.append(obj)
        if force or _stale(obj, [src] + hdrs):
            cmd = [nv] + ARCH + NVFLAGS + list(extra) + ["-c", src, "-o", obj]
            jobs.append(cmd)
    with cf.ThreadPoolExecutor(max_workers=min(8, max(1, len(jobs)))) as ex:
        for cmd, res in zip(jobs, ex.map(lambda c: subprocess.run(c, capture_output=True, text=True), jobs)):
            if res.returncode != 0:
                raise RuntimeError("nvcc failed:\n" + " ".join(cmd) + "\n" + res.stdout + res.stderr)
            if verbose and (res.stdout or res.stderr):
                print(res.stdout + res.stderr)
    if force or jobs or _stale(LIB, objs):
        tmp = LIB + ".tmp"
        cmd = [nv] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart_static", "-lrt", "-ldl", "-lpthread"]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError("link failed:\n" + " ".join(cmd) + "\n" + res.stdout + res.stderr)
        os.replace(tmp, LIB)
    build_host(force)
    return LIB


def build_host(force=False):
    """The C++ host adapter (header-only classes + C entry points), linked against libfkg.so.
    The translation units are compiled in parallel."""
    hdrs = [os.path.join(HERE, "host", "fk_mc", f) for f in os.listdir(os.path.join(HERE, "host", "fk_mc"))]
    deps = HOST_SRCS + [LIB] + hdrs + [os.path.join(ROOT, "include", f) for f in os.listdir(os.path.join(ROOT, "include"))]
    if not force and not _stale(HOST_LIB, deps):
        return HOST_LIB
    objs = [os.path.join(OUT, os.path.basename(src)[:-4] + ".host.o") for src in HOST_SRCS]
    jobs = [["g++", "-O2", "-std=c++17", "-fPIC", "-I", os.path.join(ROOT, "include"), "-c", src, "-o", obj]
            for src, obj in zip(HOST_SRCS, objs)]
    with cf.ThreadPoolExecutor(max_workers=len(jobs)) as ex:
        for cmd, res in zip(jobs, ex.map(lambda c: subprocess.run(c, capture_output=True, text=True), jobs)):
            if res.returncode != 0:
                raise RuntimeError("host adapter build failed:\n" + " ".join(cmd) + "\n" + res.stdout + res.stderr)
    tmp = HOST_LIB + ".tmp"
    cmd = ["g++", "-shared", "-o", tmp] + objs + ["-L", OUT, "-lfkg", "-Wl,-rpath,$ORIGIN"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("host adapter link failed:\n" + " ".join(cmd) + "\n" + res.stdout + res.stderr)
    os.replace(tmp, HOST_LIB)
    return HOST_LIB


if __name__ == "__main__":
    import sys
    print(build(force="--force" in sys.argv, verbose=True,
                extra=["-Xptxas", "-v"] if "--ptxas" in sys.argv else []))
