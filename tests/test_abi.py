"""The C-ABI library loads and exports every entry point include/*.h declares
(no compute calls: runs without a GPU)."""
import ctypes as C
import re
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]


def declared(header: Path) -> list[str]:
    text = header.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(tsdf_[a-z0-9_]+)\s*\(", text)))


def test_header_symbols_exported(built):
    from ros_tsdf_gb300 import _lib

    lib = C.CDLL(str(_lib.lib_path()))
    names = []
    for h in sorted((ROOT / "include").glob("*.h")):
        names += declared(h)
    assert len(names) >= 25
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_ctypes_signatures_cover_header(built):
    from ros_tsdf_gb300 import _lib

    bound = {n for n, _, _ in _lib.SIGNATURES}
    names = set()
    for h in sorted((ROOT / "include").glob("*.h")):
        names |= set(declared(h))
    assert names == bound, (names - bound, bound - names)
    _lib.load()


def test_struct_layouts_match_header(tmp_path):
    """ctypes mirrors have the size and field offsets the C compiler gives."""
    import subprocess

    from ros_tsdf_gb300 import _lib as L

    structs = {"tsdf_params": L.Params, "tsdf_engine_cfg": L.EngineCfg, "tsdf_scan_stats": L.ScanStats,
               "tsdf_scan": L.Scan, "tsdf_scan_result": L.ScanResult, "tsdf_map_info": L.MapInfo,
               "tsdf_snapshot_header": L.SnapshotHeader}
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "tsdf_c.h"', "int main(void) {"]
    for cname, py in structs.items():
        lines.append(f'  printf("{cname} size %zu\\n", sizeof({cname}));')
        for f, _ in py._fields_:
            lines.append(f'  printf("{cname} {f} %zu\\n", offsetof({cname}, {f}));')
    lines.append("  return 0; }")
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    r = subprocess.run(["gcc", f"-I{ROOT / 'include'}", str(src), "-o", str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    got = {}
    for line in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.splitlines():
        a, b, v = line.split()
        got[(a, b)] = int(v)
    for cname, py in structs.items():
        assert got[(cname, "size")] == C.sizeof(py), cname
        for f, _ in py._fields_:
            assert got[(cname, f)] == getattr(py, f).offset, (cname, f)


def test_oracle_not_linked_into_engine(built):
    """The product library must not depend on the oracle."""
    from ros_tsdf_gb300 import _lib

    data = _lib.lib_path().read_bytes()
    assert b"liboracle" not in data and b"oracle_integrate" not in data


def test_cpp_dropin_header_compiles(tmp_path):
    """include/tsdf_handler.hpp (the C++ TSDFHandler drop-in) compiles."""
    import subprocess

    src = tmp_path / "t.cpp"
    src.write_text('#include "tsdf_handler.hpp"\nint main(){ return 0; }\n')
    r = subprocess.run(["g++", "-std=c++17", "-fsyntax-only", f"-I{ROOT / 'include'}", str(src)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_cpp_pose_buffer_runs(built, tmp_path):
    """The C++ drop-in's PoseBuffer, linked against the engine library, looks up
    origins on the host (no GPU call): interpolation, latest sample, and
    std::out_of_range outside the samples."""
    import subprocess

    from ros_tsdf_gb300 import _lib

    lib = _lib.lib_path()
    src = tmp_path / "pose.cpp"
    src.write_text(r'''
#include "tsdf_handler.hpp"
#include <cstdio>
int main() {
  tsdf::PoseBuffer b(8);
  b.add(1000000000, 0.0, 0.0, 0.0);
  b.add(2000000000, 10.0, -20.0, 30.0);
  tsdf::Vector3f o = b.origin(1500000000);
  if (o(0) != 5.0f || o(1) != -10.0f || o(2) != 15.0f) return 1;
  if (b.origin(0)(2) != 30.0f || b.size() != 2) return 2;
  try { b.origin(2500000000); return 3; } catch (const std::out_of_range&) {}
  std::puts("ok");
  return 0;
}
''')
    exe = tmp_path / "pose"
    r = subprocess.run(["g++", "-std=c++17", f"-I{ROOT / 'include'}", str(src), "-o", str(exe), f"-L{lib.parent}",
                        f"-l:{lib.name}", f"-Wl,-rpath,{lib.parent}"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    run = subprocess.run([str(exe)], capture_output=True, text=True)
    assert run.returncode == 0 and run.stdout.strip() == "ok", (run.returncode, run.stderr)
