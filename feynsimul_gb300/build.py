"""Build libfeynsimul_gb300.so in-tree (nvcc, sm_103a).  ``python -m feynsimul_gb300.build``.

The device sources (csrc/fs_rng.cuh, csrc/fs_pimc.cuh) are embedded into the library as
string literals: the library specialises them per run configuration with NVRTC at
fs_create time, like the reference builds its OpenCL program from kernel.c.  Other CUDA
translation units (csrc/*.cu) are compiled into the same shared object in parallel.
"""
from __future__ import annotations

import concurrent.futures as cf
import hashlib
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libfeynsimul_gb300.so")
ROOT = os.path.dirname(PKG)

GENCODE = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", *GENCODE]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _cuda_home(nvcc: str) -> str:
    return os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))


def _embed(name: str) -> None:
    src = os.path.join(CSRC, name)
    with open(src) as f:
        text = f.read()
    delim = "FSSRC"
    assert f"){delim}\"" not in text
    out = os.path.join(BUILD, os.path.splitext(name)[0] + ".inc")
    content = f'R"{delim}(\n{text}\n){delim}"\n'
    if not os.path.exists(out) or open(out).read() != content:
        with open(out, "w") as f:
            f.write(content)


def _sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def _fingerprint(nvcc: str) -> str:
    h = hashlib.sha1()
    for d in (CSRC, os.path.join(ROOT, "include")):
        for f in sorted(os.listdir(d)):
            with open(os.path.join(d, f), "rb") as fh:
                h.update(f.encode() + fh.read())
    h.update(" ".join(NVCC_FLAGS).encode() + nvcc.encode())
    return h.hexdigest()


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    nvcc = _nvcc()
    fp = _fingerprint(nvcc)
    stamp = os.path.join(BUILD, "stamp")
    if not force and os.path.exists(LIB) and os.path.exists(stamp) and open(stamp).read() == fp:
        return LIB
    for name in ("fs_rng.cuh", "fs_pimc.cuh", "fs_mlp.cuh", "fs_batch.cuh"):
        _embed(name)
    home = _cuda_home(nvcc)
    objs = []

    def compile_one(src):
        obj = os.path.join(BUILD, os.path.basename(src) + ".o")
        cmd = [nvcc, *NVCC_FLAGS, "-I", BUILD, "-I", os.path.join(ROOT, "include"), "-c", src, "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src}:\n{r.stderr[-6000:]}")
        if verbose and r.stderr:
            print(r.stderr, file=sys.stderr)
        return obj

    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 2)) as ex:
        objs = list(ex.map(compile_one, _sources()))
    tmp = LIB + f".{os.getpid()}.tmp"
    cmd = [nvcc, *GENCODE, "-shared", "-o", tmp, *objs, "-L", os.path.join(home, "lib64"), "-lnvrtc",
           "-Xlinker", "-rpath," + os.path.join(home, "lib64")]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr[-4000:]}")
    os.replace(tmp, LIB)
    with open(stamp, "w") as f:
        f.write(fp)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
