"""CPU test of the boundary as C: a C11 program includes include/gsap.h and
include/gsap_debug.h, links libgsap.so and runs the calls that need no GPU
(configuration defaults, a refused create, a null-handle call, the debug
struct sizes)."""
import os
import shutil
import subprocess

import pytest

from conftest import ROOT

PROGRAM = r"""
#include <stdio.h>
#include <string.h>
#include "gsap.h"
#include "gsap_debug.h"

int main(void) {
    gsap_config c;
    gsap_config_default(&c);
    if (c.sort_bits != 32 || c.max_scenes != 1) return 1;
    c.sort_bits = 20;
    if (gsap_sap_create(1000, &c) != NULL) return 2;
    if (strstr(gsap_last_error(), "sort_bits") == NULL) return 3;
    uint64_t n = 0;
    if (gsap_broadphase_aabb(NULL, NULL, NULL, 10, NULL, 0, NULL, &n, GSAP_FLAG_SORTED, NULL) != GSAP_ERR_INVALID)
        return 4;
    uint32_t sizes[4];
    if (gsap_debug_sizes(sizes) != 0 || sizes[3] != 4096) return 5;
    printf("c abi ok\n");
    return 0;
}
"""


def test_header_is_c_and_links(gsap_lib, tmp_path):
    gcc = shutil.which("gcc")
    if not gcc:
        pytest.skip("needs gcc")
    from gsap_gb300 import _lib
    src = tmp_path / "abi.c"
    src.write_text(PROGRAM)
    exe = tmp_path / "abi"
    libdir = os.path.dirname(_lib.LIB_PATH)
    p = subprocess.run([gcc, "-std=c11", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"), str(src),
                        "-o", str(exe), "-L", libdir, "-l:libgsap.so", f"-Wl,-rpath,{libdir}"],
                       capture_output=True, text=True)
    assert p.returncode == 0, p.stderr
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0 and "c abi ok" in r.stdout, (r.returncode, r.stdout, r.stderr)
