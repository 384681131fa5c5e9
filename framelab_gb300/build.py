"""Builds libframelab_gb300.so in-tree with nvcc for sm_103a.

Every translation unit under csrc/ is compiled in parallel, then linked into
one shared library with the shared CUDA runtime (the same libcudart PyTorch
loads, so device pointers and streams are interchangeable).
"""
from __future__ import annotations

import hashlib
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(ROOT, "include")
OUT = os.path.join(HERE, "libframelab_gb300.so")
BUILD = os.path.join(HERE, "_build")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc() -> str:
    cand = os.environ.get("NVCC") or shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return cand


def _cuda_lib() -> str:
    nv = os.path.realpath(_nvcc())
    return os.path.join(os.path.dirname(os.path.dirname(nv)), "lib64")


def _sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC)
                  if f.endswith((".cu", ".cpp")))


def _digest(paths) -> str:
    h = hashlib.sha256()
    deps = sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC))
    deps += [os.path.join(INCLUDE, f) for f in sorted(os.listdir(INCLUDE))]
    for p in deps + [os.path.abspath(__file__)]:
        with open(p, "rb") as f:
            h.update(p.encode() + f.read())
    h.update(" ".join(ARCH).encode())
    return h.hexdigest()


# build variants: name -> (library file, object directory, extra nvcc flags)
VARIANTS = {
    "": (OUT, BUILD, ()),
    # every gather of the fast kernels checks its index, skips an access out of
    # range and counts it (fl_debug_bounds)
    "checked": (os.path.join(HERE, "libframelab_gb300_checked.so"), BUILD + "_checked",
                ("-DFL_BOUNDS_CHECK",)),
}


def variant_path(variant: str = "") -> str:
    return VARIANTS[variant][0]


def build(force: bool = False, verbose: bool = False, extra_flags=(), variant: str = "") -> str:
    out, bdir, vflags = VARIANTS[variant]
    extra_flags = (*vflags, *extra_flags)
    os.makedirs(bdir, exist_ok=True)
    stamp = os.path.join(bdir, "stamp")
    srcs = _sources()
    dig = _digest(srcs) + ":" + " ".join(extra_flags)
    if not force and os.path.exists(out) and os.path.exists(stamp):
        with open(stamp) as f:
            if f.read() == dig:
                return out
    nvcc = _nvcc()
    common = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-I", INCLUDE, "-I", CSRC,
              *ARCH, *extra_flags]

    def compile_one(src):
        obj = os.path.join(bdir, os.path.basename(src) + ".o")
        cmd = [nvcc, *common, "-c", src, "-o", obj]
        if src.endswith(".cu"):
            cmd[1:1] = ["-Xptxas", "-warn-spills", "--expt-relaxed-constexpr"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{r.stderr}")
        if verbose and r.stderr.strip():
            print(r.stderr, file=sys.stderr)
        return obj

    with ThreadPoolExecutor(max(1, min(len(srcs), os.cpu_count() or 4))) as ex:
        objs = list(ex.map(compile_one, srcs))
    tmp = out + ".tmp"
    link = [nvcc, "-shared", *ARCH, "-cudart", "shared", "-o", tmp, *objs,
            "-Xlinker", f"-rpath,{_cuda_lib()}"]
    r = subprocess.run(link, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr}")
    os.replace(tmp, out)
    with open(stamp, "w") as f:
        f.write(dig)
    return out


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
