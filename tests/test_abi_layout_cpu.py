"""The ctypes mirror of include/rtr.h (realtime_robot_gb300/__init__.py) has
the C structures' sizes and field offsets: a small C program compiled from
the header with the host compiler prints them, and each ctypes structure
must agree field by field (a mismatch would pass wrong parameters across
the boundary without any error)."""
import ctypes as C
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent

# C struct name -> (ctypes class name in the package, C field names in order)
STRUCTS = {
    "rtr_icp_params": "IcpParams",
    "rtr_icp_result": "IcpResult",
    "rtr_room_params": "RoomParams",
    "rtr_harris_params": "HarrisParams",
    "rtr_plane_params": "PlaneParams",
    "rtr_surface": "Surface",
    "rtr_recog_params": "RecogParams",
    "rtr_instance": "Instance",
    "rtr_recog_result": "RecogResult",
    "rtr_batch_pair": "BatchPair",
}


def test_ctypes_structures_match_the_header(tmp_path, rtr):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    lines = ['#include "rtr.h"', "#include <stdio.h>", "#include <stddef.h>", "int main(void) {"]
    for cname, pyname in STRUCTS.items():
        cls = getattr(rtr, pyname)
        lines.append(f'  printf("{cname} sizeof %zu\\n", sizeof({cname}));')
        for fname, _ in cls._fields_:
            lines.append(f'  printf("{cname} {fname} %zu\\n", offsetof({cname}, {fname}));')
    lines += ["  return 0;", "}"]
    src = tmp_path / "abi.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "abi"
    r = subprocess.run([cc, "-std=c11", "-I", str(ROOT / "include"), str(src), "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr  # a ctypes field the header lacks fails here
    out = {}
    for line in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.splitlines():
        s, f, v = line.split()
        out[(s, f)] = int(v)
    for cname, pyname in STRUCTS.items():
        cls = getattr(rtr, pyname)
        assert C.sizeof(cls) == out[(cname, "sizeof")], (cname, C.sizeof(cls), out[(cname, "sizeof")])
        for fname, _ in cls._fields_:
            assert getattr(cls, fname).offset == out[(cname, fname)], (cname, fname)
