"""The Python mirror agrees with include/rfgpu.h: every struct has the C
size and field offsets (a C probe compiled against the header with gcc),
and the constants have the header's values.  Host only."""
import ctypes as C
import json
import os
import re
import subprocess

import pytest

import retrofire_gb300 as rf

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "rfgpu.h")

# C struct -> (Python structure, its fields)
STRUCTS = {
    "rf_uniforms": rf.Uniforms,
    "rf_context_flags": rf.Flags,
    "rf_stats": rf.CStats,
    "rf_draw": rf.Draw,
    "rf_job": rf.Job,
    "rf_server_config": rf.ServerConfig,
    "rf_request": rf.Request,
    "rf_result": rf.Result,
}


@pytest.fixture(scope="module")
def c_layout():
    out_dir = os.path.join(ROOT, "retrofire_gb300", "_build")
    os.makedirs(out_dir, exist_ok=True)
    lines = ['#include <stddef.h>', '#include <stdio.h>', '#include "rfgpu.h"', "int main(void) {",
             '  printf("{");']
    first = True
    for cname, py in STRUCTS.items():
        parts = ['\\"size\\": %zu']
        args = ["sizeof(%s)" % cname]
        for fname, _ in py._fields_:
            parts.append('\\"%s\\": %%zu' % fname)
            args.append("offsetof(%s, %s)" % (cname, fname))
        sep = "" if first else ", "
        first = False
        lines.append('  printf("%s\\"%s\\": {%s}", %s);' % (sep, cname, ", ".join(parts), ", ".join(args)))
    lines += ['  printf("}\\n");', "  return 0;", "}"]
    src = os.path.join(out_dir, "abi_probe.c")
    exe = os.path.join(out_dir, "abi_probe")
    with open(src, "w") as f:
        f.write("\n".join(lines) + "\n")
    subprocess.check_call(["gcc", "-std=c11", "-I" + os.path.dirname(HEADER), src, "-o", exe])
    return json.loads(subprocess.check_output([exe]).decode())


@pytest.mark.parametrize("cname", list(STRUCTS))
def test_struct_layout(c_layout, cname):
    py = STRUCTS[cname]
    got = {"size": C.sizeof(py)}
    got.update({f: getattr(py, f).offset for f, _ in py._fields_})
    assert got == c_layout[cname]


def header_constants():
    src = re.sub(r"/\*.*?\*/", "", open(HEADER).read(), flags=re.S)
    consts = {m.group(1): int(m.group(2)) for m in re.finditer(r"\b(RF_[A-Z0-9_]+)\s*=\s*(\d+)", src)}
    for m in re.finditer(r"#define\s+(RF_[A-Z0-9_]+)\s+\(?(\d+)u?\b", src):
        consts[m.group(1)] = int(m.group(2))
    return consts


def test_constants_match_header():
    h = header_constants()
    mirror = {
        "RF_SHADER_FLAT": rf.FLAT, "RF_SHADER_GOURAUD": rf.GOURAUD, "RF_SHADER_TEXTURED": rf.TEXTURED,
        "RF_SHADER_TEX_GOURAUD": rf.TEX_GOURAUD, "RF_SHADER_GOURAUD_SRGB": rf.GOURAUD_SRGB,
        "RF_SAMPLER_REPEAT_POT": rf.REPEAT_POT, "RF_SAMPLER_CLAMP": rf.CLAMP, "RF_SAMPLER_ONCE": rf.ONCE,
        "RF_ARGB8888": rf.ARGB8888, "RF_XRGB8888": rf.XRGB8888, "RF_RGBA8888": rf.RGBA8888,
        "RF_BGRA8888": rf.BGRA8888,
        "RF_DEPTH_NONE": rf.DEPTH_NONE, "RF_DEPTH_LESS": rf.DEPTH_LESS, "RF_DEPTH_EQUAL": rf.DEPTH_EQUAL,
        "RF_DEPTH_GREATER": rf.DEPTH_GREATER,
        "RF_CULL_NONE": rf.CULL_NONE, "RF_CULL_BACK": rf.CULL_BACK, "RF_CULL_FRONT": rf.CULL_FRONT,
        "RF_OBJ_POSITION": rf.OBJ_POSITION, "RF_OBJ_NORMAL": rf.OBJ_NORMAL,
        "RF_OBJ_TEXCOORD": rf.OBJ_TEXCOORD, "RF_OBJ_NORMAL_TEXCOORD": rf.OBJ_NORMAL_TEXCOORD,
        "RF_DRAW_CULL_BBOX": rf.DRAW_CULL_BBOX,
    }
    for name, v in mirror.items():
        assert h[name] == v, name
    for i, st in enumerate(rf.STAGES):
        assert h["RF_STAGE_" + st.upper()] == i
    assert h["RF_STAGE_N"] == len(rf.STAGES)
    codes = {k: v for k, v in h.items() if k == "RF_OK" or k.startswith("RF_ERR_")}
    assert sorted(codes.values()) == sorted(rf.STATUS)
