"""The ctypes mirrors of the C-ABI structs (genesis_gb300/_lib.py) have the layout the C compiler
gives the declarations in include/gbmpm.h: sizes and every field offset."""

import ctypes
import os
import subprocess
import tempfile

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

STRUCTS = {
    "mpm_material": "MpmMaterial",
    "mpm_scene_config": "MpmSceneConfig",
    "mpm_pool_config": "MpmPoolConfig",
    "mpm_collider": "MpmCollider",
    "mpm_force_field": "MpmForceField",
    "mpm_diff_tool": "MpmDiffTool",
    "mpm_diff_extras": "MpmDiffExtras",
}


@pytest.mark.parametrize("c_name,py_name", sorted(STRUCTS.items()))
def test_struct_layout_matches_header(c_name, py_name):
    from genesis_gb300 import _lib

    py = getattr(_lib, py_name)
    fields = [f[0] for f in py._fields_]
    src = ["#include <stdio.h>", "#include <stddef.h>", '#include "gbmpm.h"', "int main(void) {",
           f'  printf("%zu\\n", sizeof({c_name}));']
    src += [f'  printf("%zu\\n", offsetof({c_name}, {f}));' for f in fields]
    src += ["  return 0;", "}"]
    d = tempfile.mkdtemp()
    c = os.path.join(d, "layout.c")
    exe = os.path.join(d, "layout")
    with open(c, "w") as fh:
        fh.write("\n".join(src))
    subprocess.run(["gcc", "-std=c11", "-I", INCLUDE, c, "-o", exe], check=True)
    out = [int(x) for x in subprocess.run([exe], capture_output=True, text=True, check=True).stdout.split()]
    assert out[0] == ctypes.sizeof(py), (c_name, out[0], ctypes.sizeof(py))
    for f, off in zip(fields, out[1:]):
        assert getattr(py, f).offset == off, (c_name, f)
