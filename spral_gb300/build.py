"""In-tree build of ``libspral_gb300.so`` for sm_103a (nvcc, no cmake).

Each translation unit under ``csrc/`` is compiled in parallel into
``_build/`` and linked into ``spral_gb300/libspral_gb300.so``.
"""
import concurrent.futures as cf
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
OUT = os.path.join(HERE, "libspral_gb300.so")
ROOT = os.path.dirname(HERE)
NVCC = os.environ.get("NVCC", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _sources():
    return sorted(f for f in os.listdir(CSRC) if f.endswith((".cu", ".cpp")))


def _compile(src):
    obj = os.path.join(BUILD, src + ".o")
    path = os.path.join(CSRC, src)
    deps = [path] + [os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith((".cuh", ".h"))]
    deps.append(os.path.join(ROOT, "include", "spral_ssids_gpu.h"))
    if os.path.exists(obj) and all(os.path.getmtime(obj) >= os.path.getmtime(d)
                                   for d in deps if os.path.exists(d)):
        return obj
    inc = ["-I", CSRC, "-I", os.path.join(ROOT, "include")]
    if src.endswith(".cu"):
        cmd = [NVCC, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
               "--expt-relaxed-constexpr", *inc, "-c", path, "-o", obj]
        if os.environ.get("SPRAL_GB300_PTXAS_V"):
            cmd.insert(1, "-Xptxas=-v")
    else:
        cmd = [NVCC, "-O3", "-std=c++17", "-Xcompiler", "-fPIC", *inc, "-c", path, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    if r.stderr.strip() and os.environ.get("SPRAL_GB300_VERBOSE"):
        sys.stderr.write(r.stderr)
    return obj


def build(verbose=False):
    os.makedirs(BUILD, exist_ok=True)
    srcs = _sources()
    with cf.ThreadPoolExecutor(max_workers=max(len(srcs), 1)) as ex:
        objs = list(ex.map(_compile, srcs))
    if os.path.exists(OUT) and all(os.path.getmtime(OUT) >= os.path.getmtime(o) for o in objs):
        return OUT
    cmd = [NVCC, *ARCH, "-shared", "-o", OUT, *objs, "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    if verbose:
        print(f"built {OUT}")
    return OUT


if __name__ == "__main__":
    build(verbose=True)
