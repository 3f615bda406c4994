"""In-tree build of libgsap.so for sm_103a (nvcc only, no cmake).

Each translation unit under csrc/ is compiled in parallel to _build/*.o and
linked into gsap_gb300/libgsap.so.  Objects are rebuilt when a source or a
header is newer.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import platform
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libgsap.so")
INC = os.path.join(os.path.dirname(HERE), "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# Host code: no FMA contraction, so host-side float arithmetic (the quaternion
# normalisation on upload) gives the same bits on x86 and aarch64.
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
         "--expt-relaxed-constexpr", "-Xcompiler", "-Wall", "-diag-suppress", "177"]
# The reference-model rigid-body kernels round every product and sum
# separately (no FMA contraction), as the reference's source order does.
PER_FILE = {"rigid_ref.cu": ["-fmad=false"]}


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libgsap.so")


def _sources():
    return sorted(glob.glob(os.path.join(CSRC, "*.cu")))


def _headers():
    return glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(INC, "*.h"))


def _stamp_ok() -> bool:
    """Objects built on another machine type (x86 here, aarch64 on the GPU
    box) are never reused."""
    stamp = os.path.join(BUILD, "machine.txt")
    cur = f"{platform.machine()} {nvcc()}"
    if os.path.exists(stamp) and open(stamp).read() == cur:
        return True
    for f in glob.glob(os.path.join(BUILD, "*.o")):
        os.remove(f)
    if os.path.exists(LIB):
        os.remove(LIB)
    with open(stamp, "w") as fh:
        fh.write(cur)
    return False


def build(verbose: bool = False, extra: list[str] | None = None) -> str:
    os.makedirs(BUILD, exist_ok=True)
    cc = nvcc()
    _stamp_ok()
    hdr_time = max((os.path.getmtime(h) for h in _headers()), default=0)
    jobs = []
    for src in _sources():
        obj = os.path.join(BUILD, os.path.basename(src)[:-3] + ".o")
        if (not os.path.exists(obj) or os.path.getmtime(obj) < max(os.path.getmtime(src), hdr_time)
                or extra):
            cmd = [cc, *ARCH, *FLAGS, *PER_FILE.get(os.path.basename(src), []), *(extra or []), "-I", INC,
                   "-c", src, "-o", obj]
            jobs.append((src, cmd))

    def run(job):
        src, cmd = job
        p = subprocess.run(cmd, capture_output=True, text=True)
        if p.returncode != 0:
            raise RuntimeError(f"nvcc failed for {os.path.basename(src)}:\n{p.stderr}")
        if verbose and p.stderr.strip():
            print(p.stderr)
        return src

    with cf.ThreadPoolExecutor(max_workers=min(8, max(1, len(jobs)))) as ex:
        list(ex.map(run, jobs))
    objs = [os.path.join(BUILD, os.path.basename(s)[:-3] + ".o") for s in _sources()]
    if jobs or not os.path.exists(LIB):
        cmd = [cc, *ARCH, "-shared", "-o", LIB, *objs, "-lcudart_static", "-lrt", "-ldl", "-lpthread"]
        p = subprocess.run(cmd, capture_output=True, text=True)
        if p.returncode != 0:
            raise RuntimeError(f"link failed:\n{p.stderr}")
    return LIB


if __name__ == "__main__":
    print(build(verbose=True))
