"""The Python mirror's ctypes structures have the C header's layout: a C program built with gcc
against include/p9idg.h prints sizeof and offsetof of every field of every struct the ABI passes,
and each must equal the ctypes structure's (a mismatch would make the library read or write the
wrong bytes of a caller's struct)."""
import ctypes
import os
import shutil
import subprocess

import pytest

from conftest import ROOT, pkg

deconv = pkg.deconv
idg = pkg.idg

# C struct -> (ctypes structure, {ctypes field name: C field name} where they differ)
STRUCTS = {
    "p9idg_params": (pkg._native.Params, {}),
    "p9idg_subgrid": (pkg._native.SubgridC, {}),
    "p9idg_plan_info": (pkg._native.PlanInfo, {}),
    "p9idg_tuning": (idg.Tuning, {}),
    "p9idg_cd_result": (deconv._CdResult, {}),
    "p9idg_mc_params": (deconv.McParams, {"lambda_": "lambda"}),
    "p9idg_mc_cycle": (deconv.McCycle, {}),
}


def test_ctypes_structures_match_the_header(tmp_path):
    gcc = shutil.which("gcc")
    if not gcc:
        pytest.skip("no C compiler")
    lines = ["#include <stddef.h>", "#include <stdio.h>", '#include "p9idg.h"', "int main(void) {"]
    for cname, (cls, rename) in STRUCTS.items():
        lines.append(f'    printf("{cname} size %zu\\n", sizeof({cname}));')
        for fname, _ in cls._fields_:
            cf = rename.get(fname, fname)
            lines.append(f'    printf("{cname} {fname} %zu\\n", offsetof({cname}, {cf}));')
    lines += ["    return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.run([gcc, "-std=c99", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)],
                   check=True, capture_output=True, text=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split("\n")
    got = {tuple(l.split()[:2]): int(l.split()[2]) for l in out if l.strip()}
    for cname, (cls, _) in STRUCTS.items():
        assert got[(cname, "size")] == ctypes.sizeof(cls), cname
        for fname, _ in cls._fields_:
            assert got[(cname, fname)] == getattr(cls, fname).offset, (cname, fname)
