"""In-tree build of the native libraries (nvcc / g++, no cmake).

libtsdf_gb300.so  the engine: CUDA kernels for sm_103a + host engine + C-ABI
libscangen.so     seeded synthetic lidar scans (host C++)

Outputs go to ros_tsdf_gb300/lib/.  A library is rebuilt when a source is
newer than it, or when it was built for another machine architecture.
"""
from __future__ import annotations

import os
import platform
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
LIB = PKG / "lib"
INCLUDE = PKG.parent / "include"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-fno-fast-math"]
KERNEL_FLAGS = ["-fmad=false", "-prec-div=true", "-prec-sqrt=true", "-ftz=false"]
CXX_FLAGS = ["-O3", "-std=c++17", "-fPIC", "-ffp-contract=off", "-fno-fast-math", "-Wall", "-pthread"]


def _nvcc() -> str:
    for c in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _stamp_ok(out: Path, srcs: list[Path]) -> bool:
    stamp = out.with_suffix(out.suffix + ".arch")
    if not out.exists() or not stamp.exists():
        return False
    if stamp.read_text().strip() != platform.machine():
        return False
    t = out.stat().st_mtime
    return all(s.stat().st_mtime <= t for s in srcs)


def _write_stamp(out: Path) -> None:
    out.with_suffix(out.suffix + ".arch").write_text(platform.machine() + "\n")


def _run_all(cmds: list[list[str]], verbose: bool) -> None:
    procs = []
    for c in cmds:
        if verbose:
            print(" ".join(c), file=sys.stderr)
        procs.append((c, subprocess.Popen(c, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
    errs = []
    for c, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            errs.append(f"$ {' '.join(c)}\n{out.decode(errors='replace')}")
        elif verbose and out:
            print(out.decode(errors="replace"), file=sys.stderr)
    if errs:
        raise RuntimeError("native build failed:\n" + "\n".join(errs))


def build(verbose: bool = False, force: bool = False) -> dict:
    LIB.mkdir(exist_ok=True)
    nvcc = _nvcc()
    eng = LIB / "libtsdf_gb300.so"
    gen = LIB / "libscangen.so"
    eng_srcs = [CSRC / "tsdf_kernels.cu", CSRC / "tsdf_engine.cu", CSRC / "tsdf_blocks.cu", CSRC / "tsdf_internal.h",
                INCLUDE / "tsdf_c.h"]
    gen_srcs = [CSRC / "scangen.cpp"]
    build_dir = LIB / "_obj"
    build_dir.mkdir(exist_ok=True)
    stage1 = []
    need_eng = force or not _stamp_ok(eng, eng_srcs)
    need_gen = force or not _stamp_ok(gen, gen_srcs)
    if need_eng:
        stage1.append([nvcc, *ARCH, *NVCC_FLAGS, *KERNEL_FLAGS, "-c", str(CSRC / "tsdf_kernels.cu"),
                       "-o", str(build_dir / "tsdf_kernels.o")])
        stage1.append([nvcc, *ARCH, *NVCC_FLAGS, "-c", str(CSRC / "tsdf_engine.cu"),
                       "-o", str(build_dir / "tsdf_engine.o")])
        stage1.append([nvcc, *ARCH, *NVCC_FLAGS, *KERNEL_FLAGS, "-c", str(CSRC / "tsdf_blocks.cu"),
                       "-o", str(build_dir / "tsdf_blocks.o")])
    if need_gen:
        stage1.append(["g++", *CXX_FLAGS, "-shared", "-o", str(gen), str(CSRC / "scangen.cpp")])
    _run_all(stage1, verbose)
    if need_eng:
        _run_all([[nvcc, *ARCH, "-shared", "-o", str(eng), str(build_dir / "tsdf_kernels.o"),
                   str(build_dir / "tsdf_engine.o"), str(build_dir / "tsdf_blocks.o"), "-lcudart", "-lpthread"]], verbose)
        _write_stamp(eng)
    if need_gen:
        _write_stamp(gen)
    return {"engine": str(eng), "scangen": str(gen)}


if __name__ == "__main__":
    print(build(verbose=True, force="--force" in sys.argv))
