"""ros_tsdf's own integration code run as host code (TEST INFRASTRUCTURE ONLY).

Recipe and driver for the reference-side parity harness:

* ``generate()`` reads ros_tsdf's sources where they lie (REF_ROOT) and writes
  a copy into oracle/_ref/ (git-ignored, never committed) in which the only
  change is that every kernel launch ``K<<<g, b>>>(args)`` becomes
  ``ref_launch(g, b, K)(args)``, on the same line.  The two headers are
  copied unchanged.
* ``build()`` compiles oracle/ref_harness.cpp over that copy with the host
  stand-ins in oracle/ref_shim/ (CUDA runtime, Eigen Vector3f, PCL types,
  assert) into two programs: ``ref_run_powf`` (the reference's ``pow(x, 2)``
  as the float square, the semantics its device code has) and
  ``ref_run_powd`` (the C++ library's ``pow(float, int)``, which promotes to
  double: its semantics as host code).  Flags: ``-ffp-contract=off`` (no FMA,
  like the oracle and the engine; nvcc would contract the reference's device
  code by default) and ``-fwrapv`` (the hash's int multiply wraps as it does on
  the GPU).  A machine without the reference sources rebuilds the
  programs from the generated copy when it travelled with the repository.
* ``run()`` feeds scans to a program in a subprocess (a crash in reference code
  cannot take the caller down) and parses what it wrote.

Only tests/ and the CPU legs of bench.py use this module; the product never
imports it.
"""
from __future__ import annotations

import os
import platform
import re
import struct
import subprocess
import tempfile
from dataclasses import dataclass, field
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
OUT = HERE / "_ref"
SHIM = HERE / "ref_shim"
HARNESS = HERE / "ref_harness.cpp"
REF_ROOT = Path(os.environ.get("TSDF_REFERENCE_ROOT", "/root/reference"))

# reference file (relative to REF_ROOT) -> generated file (relative to OUT)
FILES = {
    "tsdf_package/src/cuda/tsdf_handler.cu": "src/tsdf_handler_host.cc",
    "tsdf_package/src/cuda/tsdf_container.cu": "src/tsdf_container_host.cc",
    "tsdf_package/include/cuda/tsdf_handler.cuh": "include/cuda/tsdf_handler.cuh",
    "tsdf_package/include/cuda/tsdf_container.cuh": "include/cuda/tsdf_container.cuh",
}
# tsdf_handler.cu launches kernels at lines 702, 821, 1078, 1083, 1134, 1142,
# 1172, 1204, 1256 and 1264.
EXPECTED_LAUNCHES = 10
_LAUNCH = re.compile(r"\b([A-Za-z_]\w*)\s*<<<(.*?)>>>")

VARIANTS = {"float": ["-DREF_POW_FLOAT"], "double": []}
PROGRAMS = {"float": OUT / "ref_run_powf", "double": OUT / "ref_run_powd"}
CXXFLAGS = ["-O2", "-std=c++17", "-ffp-contract=off", "-fno-fast-math", "-fwrapv", "-w", "-pthread"]

NUM_HEAP_BLOCKS = 524288        # tsdf_container.cuh:31
HASH_TABLE_SIZE = 4 * 131072    # tsdf_container.cuh:23-27
PUBLISH_VOXELS_MAX_SIZE = 400000  # tsdf_handler.cuh:16
GC_QUEUE_MAX = 1000             # tsdf_handler.cuh:20

FLAG_INTEGRATE, FLAG_STAGES, FLAG_NO_PUBLISH_DATA = 1, 2, 4
STATUS_GC_QUEUE_OVERFLOW = 4


def generate() -> bool:
    """Write the launch-rewritten copy of the reference into oracle/_ref/.

    Returns False when the reference sources are not on this machine."""
    if not all((REF_ROOT / k).exists() for k in FILES):
        return False
    launches = 0
    for src, dst in FILES.items():
        text = (REF_ROOT / src).read_text()
        if src.endswith(".cu"):
            text, n = _LAUNCH.subn(lambda m: f"ref_launch({m.group(2)}, {m.group(1)})", text)
            launches += n
        out = OUT / dst
        out.parent.mkdir(parents=True, exist_ok=True)
        if not out.exists() or out.read_text() != text:
            out.write_text(text)
    if launches != EXPECTED_LAUNCHES:
        raise RuntimeError(f"expected {EXPECTED_LAUNCHES} kernel launches in the reference, rewrote {launches}")
    return True


def _generated() -> bool:
    return all((OUT / v).exists() for v in FILES.values())


def _stale(prog: Path, srcs: list[Path]) -> bool:
    stamp = prog.with_name(prog.name + ".arch")
    if not prog.exists() or not stamp.exists() or stamp.read_text().strip() != platform.machine():
        return True
    t = prog.stat().st_mtime
    return any(s.stat().st_mtime > t for s in srcs)


def build(verbose: bool = False) -> bool:
    """Generate (when the reference is present) and compile both programs.

    Returns False when neither the reference nor a generated copy exists."""
    generate()
    if not _generated():
        return False
    srcs = [HARNESS, *SHIM.rglob("*"), *(OUT / v for v in FILES.values())]
    srcs = [s for s in srcs if s.is_file()]
    procs = []
    for name, defs in VARIANTS.items():
        prog = PROGRAMS[name]
        if not _stale(prog, srcs):
            continue
        cmd = ["g++", *CXXFLAGS, *defs, "-I", str(SHIM), "-I", str(OUT / "include"), "-I", str(OUT / "src"),
               str(HARNESS), "-o", str(prog)]
        if verbose:
            print(" ".join(cmd))
        procs.append((prog, cmd, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
    for prog, cmd, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            raise RuntimeError(f"reference harness build failed:\n$ {' '.join(cmd)}\n{out.decode(errors='replace')}")
        prog.with_name(prog.name + ".arch").write_text(platform.machine() + "\n")
    return True


def available(pow_mode: str = "float") -> bool:
    p = PROGRAMS[pow_mode]
    stamp = p.with_name(p.name + ".arch")
    return p.exists() and stamp.exists() and stamp.read_text().strip() == platform.machine()


# ---- running ---------------------------------------------------------------


@dataclass
class ScanOut:
    status: int
    count: int
    seconds: float
    below_heap: int   # voxels of heap block -1 written (updates whose block is missing)
    pos: np.ndarray   # (kept, 3) float32
    data: np.ndarray  # (kept, 2) float32 {sdf, weight}


@dataclass
class StateDump:
    scan: int
    block_count: int
    entry_index: np.ndarray  # (E,) int32 hash-entry index
    centre: np.ndarray       # (E, 3) float32 block centre
    offset: np.ndarray       # (E,) int32 chain offset
    heap_pos: np.ndarray     # (E,) int32 block heap slot
    voxels: np.ndarray       # (E, 512, 2) float32
    free_blocks: np.ndarray  # (NUM_HEAP_BLOCKS,) int32


@dataclass
class PointStages:
    segment: np.ndarray        # (6,) start xyz, end xyz
    block_cells: np.ndarray    # (nb, 3) float32 centres
    voxel_cells: np.ndarray    # (nv, 3) float32 centres
    local: np.ndarray          # (nv,) int32
    dist: np.ndarray           # (nv,) float32
    weight: np.ndarray         # (nv,) float32


@dataclass
class RefResult:
    scans: list = field(default_factory=list)    # ScanOut per integrated scan
    dumps: dict = field(default_factory=dict)    # scan index -> StateDump
    stages: dict = field(default_factory=dict)   # scan index -> [PointStages]
    assert_failures: int = 0


def _write_input(path: Path, params, scans, flags: int, dump_after, stage_scans) -> None:
    with open(path, "wb") as f:
        f.write(b"TSDFREF1")
        f.write(struct.pack("<5f", params.voxel_size, params.truncation_distance, params.max_weight,
                            params.publish_distance_squared, params.garbage_collect_distance_squared))
        f.write(struct.pack("<ii", flags, len(scans)))
        for xyz, org in scans:
            a = np.ascontiguousarray(np.asarray(xyz, np.float32)[:, :3])
            f.write(struct.pack("<i", a.shape[0]))
            f.write(np.asarray(org, np.float32).reshape(3).tobytes())
            f.write(a.tobytes())
        for lst in (dump_after, stage_scans):
            f.write(struct.pack("<i", len(lst)))
            f.write(np.asarray(list(lst), np.int32).tobytes())


class _Buf:
    def __init__(self, b: bytes):
        self.b = b
        self.o = 0

    def take(self, dtype, n: int) -> np.ndarray:
        dt = np.dtype(dtype)
        a = np.frombuffer(self.b, dt, n, self.o)
        self.o += dt.itemsize * n
        return a

    def i32(self) -> int:
        return int(self.take("<i4", 1)[0])


def _parse(b: bytes) -> RefResult:
    if b[:8] != b"TSDFREFO":
        raise RuntimeError("reference harness wrote no output header")
    r = _Buf(b)
    r.o = 8
    res = RefResult()
    while True:
        tag = r.i32()
        if tag == 1:
            _k, status, count = r.i32(), r.i32(), r.i32()
            secs = float(r.take("<f8", 1)[0])
            below = r.i32()
            kept = r.i32()
            q = r.take("<f4", kept * 5).reshape(kept, 5)
            res.scans.append(ScanOut(status, count, secs, below, q[:, :3].copy(), q[:, 3:].copy()))
        elif tag == 2:
            scan, bc, e = r.i32(), r.i32(), r.i32()
            rec = r.take([("i", "<i4"), ("c", "<f4", 3), ("o", "<i4"), ("h", "<i4")], e)
            vox = r.take("<f4", e * 1024).reshape(e, 512, 2)
            fb = r.take("<i4", NUM_HEAP_BLOCKS)
            res.dumps[scan] = StateDump(scan, bc, rec["i"].copy(), rec["c"].copy(), rec["o"].copy(), rec["h"].copy(),
                                        vox.copy(), fb.copy())
        elif tag == 3:
            scan, n = r.i32(), r.i32()
            pts = []
            for _ in range(n):
                seg = r.take("<f4", 6).copy()
                nb = r.i32()
                bcells = r.take("<f4", nb * 3).reshape(nb, 3).copy()
                nv = r.i32()
                rec = r.take([("c", "<f4", 3), ("l", "<i4"), ("d", "<f4"), ("w", "<f4")], nv)
                pts.append(PointStages(seg, bcells, rec["c"].copy(), rec["l"].copy(), rec["d"].copy(), rec["w"].copy()))
            res.stages[scan] = pts
        elif tag == 9:
            res.assert_failures = int(r.take("<i8", 1)[0])
            return res
        else:
            raise RuntimeError(f"reference harness output: unknown record tag {tag}")


def run(params, scans, *, pow_mode: str = "float", integrate: bool = True, dump_after=(), stage_scans=(),
        publish_data: bool = True, timeout: float = 1800.0) -> RefResult:
    """Run ros_tsdf's integration call on scans [(xyz (n,3), origin (3,)), ...].

    One TSDFHandler for all scans, as one ROS node holds one.  Each scan is one
    processPointCloudAndUpdateVoxels call with the publish count zeroed on
    entry.  dump_after: scans after which the whole hash table, the voxels of
    every allocated block and the heap's free list are returned.
    stage_scans: scans whose per-point stages (segment, DDA cells, local
    index, distance and weight updates) are returned."""
    prog = PROGRAMS[pow_mode]
    if not available(pow_mode):
        raise RuntimeError(f"{prog} is not built for this machine (oracle.ref.build())")
    flags = (FLAG_INTEGRATE if integrate else 0) | (0 if publish_data else FLAG_NO_PUBLISH_DATA)
    with tempfile.TemporaryDirectory(prefix="tsdf_ref_") as td:
        inp, out = Path(td) / "in.bin", Path(td) / "out.bin"
        _write_input(inp, params, scans, flags, dump_after, stage_scans)
        p = subprocess.run([str(prog), str(inp), str(out)], capture_output=True, text=True, timeout=timeout)
        if p.returncode != 0:
            raise RuntimeError(f"reference harness exited {p.returncode}: {p.stderr[-2000:]}")
        return _parse(out.read_bytes())


# ---- conversions to the oracle's representation ------------------------------


def centre_to_key(centre: np.ndarray, size: float) -> np.ndarray:
    """Integer cell coordinates of float cell centres floor(x/s)/(1/s) + s/2
    (tsdf_handler.cu:65-85): exact for |key| < 2^20."""
    c = np.asarray(centre, np.float64)
    return np.rint((c - size / 2.0) / size).astype(np.int64)


# ---- timing (the CPU legs of bench.py) ----------------------------------------

BYTES_PER_PROCESS = 7 << 30  # the reference's fixed heap twice (host and "device" copy) plus the hash table


def concurrency(n_jobs: int) -> int:
    """Processes to run at once: one per host core, bounded by the host memory
    each reference process needs (its 524288-block heap is allocated twice)."""
    cores = os.cpu_count() or 1
    avail = None
    try:
        for line in Path("/proc/meminfo").read_text().splitlines():
            if line.startswith("MemAvailable:"):
                avail = int(line.split()[1]) * 1024
    except OSError:
        pass
    by_mem = max(1, int(0.75 * avail) // BYTES_PER_PROCESS) if avail else 1
    return max(1, min(cores, n_jobs, by_mem))


def run_many(jobs, *, procs: int | None = None, pow_mode: str = "float", timeout: float = 1800.0):
    """Run several maps, one reference process per map, at most `procs` at a
    time.  jobs: [(params, scans)].  Returns ([RefResult per job], procs).
    Publish data is not returned (counts and per-scan seconds are)."""
    prog = PROGRAMS[pow_mode]
    if not available(pow_mode):
        raise RuntimeError(f"{prog} is not built for this machine (oracle.ref.build())")
    procs = procs or concurrency(len(jobs))
    results: list = [None] * len(jobs)
    with tempfile.TemporaryDirectory(prefix="tsdf_ref_") as td:
        pending = list(range(len(jobs)))
        running: list = []
        while pending or running:
            while pending and len(running) < procs:
                j = pending.pop(0)
                params, scans = jobs[j]
                inp, out = Path(td) / f"in{j}.bin", Path(td) / f"out{j}.bin"
                _write_input(inp, params, scans, FLAG_INTEGRATE | FLAG_NO_PUBLISH_DATA, (), ())
                p = subprocess.Popen([str(prog), str(inp), str(out)], stdout=subprocess.DEVNULL,
                                     stderr=subprocess.PIPE, text=True)
                running.append((j, p, out))
            j, p, out = running.pop(0)
            _, err = p.communicate(timeout=timeout)
            if p.returncode != 0:
                for _, q, _ in running:
                    q.kill()
                raise RuntimeError(f"reference harness exited {p.returncode}: {err[-2000:]}")
            results[j] = _parse(out.read_bytes())
    return results, procs
