"""Build recipe of librtmc.so (in-tree, sm_103a only).

Translation units compiled in parallel: the transport kernel family (kernels.cu over
transport.cuh, compiled once per precision and kernel group: transport, batched,
adjoint, split schedule), the slice fold (fold.cu) and the static scratch (noalloc.cu) with nvcc for
sm_103a, the host table builder and the context/C-ABI with g++; linked by nvcc into
radiativetransfermontecarlo_gb300/librtmc.so with the CUDA runtime linked statically.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = PKG / "librtmc.so"
ARCH = "-gencode=arch=compute_103a,code=sm_103a"


def _cuda_home() -> Path:
    for c in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if c and (Path(c) / "bin" / "nvcc").exists():
            return Path(c)
    nvcc = shutil.which("nvcc")
    if nvcc:
        return Path(nvcc).resolve().parent.parent
    raise RuntimeError("nvcc not found: set CUDA_HOME")


def _sources():
    return sorted(CSRC.glob("*.cu")) + sorted(CSRC.glob("*.cpp")) + sorted(CSRC.glob("*.h")) + sorted(CSRC.glob("*.cuh")) + [PKG.parent / "include" / "rtmc.h"]


def up_to_date() -> bool:
    if not LIB.exists():
        return False
    t = LIB.stat().st_mtime
    return all(s.stat().st_mtime <= t for s in _sources())


def build(verbose: bool = False, force: bool = False, ptxas_info: bool = False) -> Path:
    if not force and up_to_date():
        return LIB
    cuda = _cuda_home()
    nvcc = str(cuda / "bin" / "nvcc")
    BUILD.mkdir(exist_ok=True)
    inc = [f"-I{cuda / 'include'}", f"-I{PKG.parent / 'include'}"]
    jobs = []
    objs = []
    units = []
    for cu in sorted(CSRC.glob("*.cu")):
        if cu.name == "kernels.cu":
            for real, suf in (("float", "f32"), ("double", "f64")):
                for part in (1, 2, 3, 4):
                    units.append((cu, f"kernels_{suf}_{part}", [f"-DRTMC_REAL={real}", f"-DRTMC_SUFFIX={suf}",
                                                                 f"-DRTMC_PART={part}"]))
        else:
            units.append((cu, cu.stem, []))
    extra = os.environ.get("RTMC_NVCC_EXTRA", "").split()  # e.g. -DRTMC_TRANSPORT_MIN_BLOCKS=3
    for cu, stem, defs in units:
        o = BUILD / (stem + ".o")
        cmd = [nvcc, ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", *defs, *extra, *inc, "-c", str(cu),
               "-o", str(o)]
        if ptxas_info:
            cmd.insert(2, "-Xptxas=-v")
        jobs.append(cmd)
        objs.append(o)
    for cpp in sorted(CSRC.glob("*.cpp")):
        o = BUILD / (cpp.stem + ".o")
        jobs.append(["g++", "-O2", "-std=c++17", "-fPIC", "-Wall", *inc, "-c", str(cpp), "-o", str(o)])
        objs.append(o)
    procs = [subprocess.Popen(c, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True) for c in jobs]
    errs = []
    for c, p in zip(jobs, procs):
        out, _ = p.communicate()
        if verbose or ptxas_info or p.returncode:
            sys.stderr.write(out)
        if p.returncode:
            errs.append(" ".join(c))
    if errs:
        raise RuntimeError("librtmc build failed:\n" + "\n".join(errs))
    tmp = LIB.with_suffix(".so.tmp")
    link = [nvcc, ARCH, "-shared", "-Xcompiler", "-fPIC", *map(str, objs), "-o", str(tmp), "-lpthread", "-ldl", "-lrt"]
    r = subprocess.run(link, capture_output=True, text=True)
    if r.returncode:
        raise RuntimeError("librtmc link failed:\n" + r.stdout + r.stderr)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    build(verbose=True, force="--force" in sys.argv, ptxas_info="--ptxas" in sys.argv)
    print(LIB)
